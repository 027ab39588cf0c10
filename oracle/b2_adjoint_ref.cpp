/*
 * b2_adjoint_ref.cpp — host reference for the differentiable step (test infrastructure only:
 * the tests load it to check the GPU backward pass; nothing in the library links it).
 *
 * Input is a tape exported by b2g_tape_get_step plus the bodies' mass data. Three runs:
 *   replay_f32   the taped solver steps re-run sequentially in f32, colour by colour, with the
 *                templated forward functions of the differentiable step; records every
 *                discrete decision (friction/normal clamp states, block-solver case and
 *                reduction, restitution triggers, translation/rotation and position-correction
 *                clamps). Its result must equal the GPU's recorded final state bit for bit.
 *   forward_f64  the same steps in f64 with those decisions frozen: the function whose central
 *                finite differences the gradients are checked against.
 *   backward_f64 the reverse pass in f64 (sequential; the same reverse order as the GPU).
 * The solver steps follow B2island::solve (private/dynamics/b2_island_private.rs:129-328) and
 * B2contactSolver (private/dynamics/b2_contact_solver_private.rs:20-730).
 */
#include <cstdint>
#include <cstring>
#include <vector>

#include "../box2d-rs_gb300/csrc/b2g_adjoint.cuh"

using namespace b2g::adj;

namespace {

struct HSlot {
    int32_t idx[4];
    float geo[4], lp[4], inv[4], lc[4], mat[4], rad[4], imp[4];
    int32_t carry[4];
};
static_assert(sizeof(HSlot) == 144, "b2g_tape_slot layout");
struct HStep {
    float dt, dt_ratio, gx, gy;
    int32_t vi, pi, warm, nslots;
    int64_t slot_off;
    int32_t ncol, ncontacts;
};
static_assert(sizeof(HStep) == 48, "b2g_tape_step layout");

template <class T>
struct Body {
    P2<T> c, v;
    T a, w;
};

struct Ref {
    int nb = 0;
    std::vector<BodyStatic> bs;
    int T = 0;
    std::vector<HStep> steps;
    std::vector<std::vector<int>> col;
    std::vector<std::vector<HSlot>> slots;
    /* decisions of the f32 replay */
    std::vector<std::vector<VelDecision>> vdec;       /* [t][it * ns + k] */
    std::vector<std::vector<unsigned char>> pdec;     /* [t][(it * ns + k) * 2 + j] */
    std::vector<std::vector<unsigned char>> clamp;    /* [t][b] */
    std::vector<std::vector<int>> vcount, bias;       /* [t][k], [t][2k + j] */
    bool have_dec = false;
    long long carry_mismatch = 0;                     /* f32 replay: carried impulse != recorded one */
    /* the f32 replay's trajectory: each step's starting state and the impulses carried into it, the
     * points an anchored f64 pass linearises around */
    std::vector<std::vector<Body<float>>> anchor_start;
    std::vector<std::vector<float>> anchor_end_prev;
};

template <class T>
struct Trace {
    std::vector<std::vector<Body<T>>> start, vel1, vel2;  /* [t][b] */
    std::vector<std::vector<T>> wv;                       /* [t][(it * ns + k) * 10] */
    std::vector<std::vector<T>> ww;                       /* [t][k * 6] */
    std::vector<std::vector<T>> wp;                       /* [t][(it * ns + k) * 6] */
    std::vector<std::vector<T>> imp0;                     /* [t][4k]: impulses entering the warm start */
};

SlotStatic slot_static(const HSlot& t) {
    SlotStatic s{};
    s.a = t.idx[0];
    s.b = t.idx[1];
    s.count = t.idx[2] & 0xff;
    s.mtype = (t.idx[2] >> 8) & 0xff;
    s.flags = (t.idx[2] >> 16) & 3;
    s.colour = t.idx[3];
    int isl;
    std::memcpy(&isl, &t.rad[2], 4);
    s.island = isl;
    s.carry[0] = t.carry[0];
    s.carry[1] = t.carry[1];
    for (int i = 0; i < 2; ++i) {
        s.ln[i] = t.geo[i];
        s.lpt[i] = t.geo[2 + i];
    }
    for (int i = 0; i < 4; ++i) s.lp[i] = t.lp[i];
    s.mA = t.inv[0];
    s.mB = t.inv[1];
    s.iA = t.inv[2];
    s.iB = t.inv[3];
    s.rA = t.rad[0];
    s.rB = t.rad[1];
    s.friction = t.mat[0];
    s.restitution = t.mat[1];
    s.threshold = t.mat[2];
    return s;
}
int pos_iters(const HSlot& t) {
    int n;
    std::memcpy(&n, &t.rad[3], 4);
    return n;
}

/* The taped steps. frozen = false: the f32 replay, which records every decision and its own
 * trajectory; frozen = true: the frozen-decision model (any T). anchored (with frozen): every step
 * starts from the f32 replay's state and carried impulses instead of the previous step's result, so a
 * reverse pass over the trace is the f64-accurate gradient of the f32 trajectory's linearisation. */
template <class T>
void forward(Ref& R, bool frozen, std::vector<Body<T>>& st, Trace<T>* tr, bool anchored = false) {
    if (!frozen) {
        R.vdec.assign(R.T, {});
        R.pdec.assign(R.T, {});
        R.clamp.assign(R.T, {});
        R.vcount.assign(R.T, {});
        R.bias.assign(R.T, {});
    }
    if (!frozen) R.carry_mismatch = 0;
    std::vector<T> end_prev;  /* impulses each slot of the previous step stored */
    if (tr) {
        tr->imp0.assign(R.T, {});
        tr->start.assign(R.T, {});
        tr->vel1.assign(R.T, {});
        tr->vel2.assign(R.T, {});
        tr->wv.assign(R.T, {});
        tr->ww.assign(R.T, {});
        tr->wp.assign(R.T, {});
    }
    if (!frozen) {
        R.anchor_start.assign(R.T, {});
        R.anchor_end_prev.assign(R.T, {});
    }
    for (int t = 0; t < R.T; ++t) {
        const HStep& sp = R.steps[t];
        const std::vector<HSlot>& sl = R.slots[t];
        const std::vector<int>& co = R.col[t];
        const int ns = sp.nslots, ncol = sp.ncol;
        const T h = (T)sp.dt;
        if (!frozen) {
            R.anchor_start[t].resize(R.nb);
            for (int b = 0; b < R.nb; ++b) {
                Body<float>& a = R.anchor_start[t][b];
                a.c = p2((float)st[b].c.x, (float)st[b].c.y);
                a.a = (float)st[b].a;
                a.v = p2((float)st[b].v.x, (float)st[b].v.y);
                a.w = (float)st[b].w;
            }
            R.anchor_end_prev[t].assign(end_prev.begin(), end_prev.end());
        } else if (anchored) {
            for (int b = 0; b < R.nb; ++b) {
                const Body<float>& a = R.anchor_start[t][b];
                st[b].c = p2((T)a.c.x, (T)a.c.y);
                st[b].a = (T)a.a;
                st[b].v = p2((T)a.v.x, (T)a.v.y);
                st[b].w = (T)a.w;
            }
            end_prev.assign(R.anchor_end_prev[t].begin(), R.anchor_end_prev[t].end());
        }
        if (tr) tr->start[t] = st;
        for (int b = 0; b < R.nb; ++b)
            if (R.bs[b].type == 2) integrate_velocity(R.bs[b], h, (T)sp.gx, (T)sp.gy, st[b].v, st[b].w);
        if (tr) tr->vel1[t] = st;
        std::vector<VC<T>> vc(ns);
        std::vector<T> imp(4 * (size_t)ns, (T)0), raw(4 * (size_t)ns, (T)0);
        if (!frozen) {
            R.vcount[t].assign(ns, 0);
            R.bias[t].assign(2 * (size_t)ns, 0);
        }
        for (int k = 0; k < ns; ++k) {
            const SlotStatic ss = slot_static(sl[k]);
            const P2<T> lcA = p2((T)sl[k].lc[0], (T)sl[k].lc[1]), lcB = p2((T)sl[k].lc[2], (T)sl[k].lc[3]);
            if (frozen) {
                vc[k].vcount = R.vcount[t][k];
                vc[k].bias_on[0] = R.bias[t][2 * k];
                vc[k].bias_on[1] = R.bias[t][2 * k + 1];
            }
            init_slot(ss, st[ss.a].c, st[ss.a].a, st[ss.b].c, st[ss.b].a, st[ss.a].v, st[ss.a].w, st[ss.b].v,
                      st[ss.b].w, lcA, lcB, vc[k], frozen);
            if (!frozen) {
                R.vcount[t][k] = vc[k].vcount;
                R.bias[t][2 * k] = vc[k].bias_on[0];
                R.bias[t][2 * k + 1] = vc[k].bias_on[1];
            }
            /* the impulses carried into the step: the previous step's stored impulse of the
             * matched point (b2_contact.rs:277-298), else the recorded value */
            for (int j = 0; j < 2; ++j) {
                T n = (T)sl[k].imp[2 * j], tg = (T)sl[k].imp[2 * j + 1];
                const int cj = j < ss.count ? ss.carry[j] : -1;
                if (t > 0 && cj >= 0) {
                    n = end_prev[2 * (size_t)cj];
                    tg = end_prev[2 * (size_t)cj + 1];
                    if (!frozen && !(n == (T)sl[k].imp[2 * j] && tg == (T)sl[k].imp[2 * j + 1])) ++R.carry_mismatch;
                }
                raw[4 * k + 2 * j] = n;
                raw[4 * k + 2 * j + 1] = tg;
            }
            if (sp.warm) {
                imp[4 * k] = (T)sp.dt_ratio * raw[4 * k];
                imp[4 * k + 1] = (T)sp.dt_ratio * raw[4 * k + 1];
                if (ss.count > 1) {
                    imp[4 * k + 2] = (T)sp.dt_ratio * raw[4 * k + 2];
                    imp[4 * k + 3] = (T)sp.dt_ratio * raw[4 * k + 3];
                }
            }
        }
        if (tr) tr->imp0[t] = imp;
        if (tr) tr->ww[t].assign(6 * (size_t)ns, (T)0);
        if (sp.warm) {
            for (int c = 0; c < ncol; ++c)
                for (int k = co[c]; k < co[c + 1]; ++k) {
                    const SlotStatic ss = slot_static(sl[k]);
                    Body<T> A = st[ss.a], B = st[ss.b];
                    if (tr) {
                        T* r = &tr->ww[t][6 * (size_t)k];
                        r[0] = A.v.x; r[1] = A.v.y; r[2] = A.w; r[3] = B.v.x; r[4] = B.v.y; r[5] = B.w;
                    }
                    const T ni[2] = {imp[4 * k], imp[4 * k + 2]}, ti[2] = {imp[4 * k + 1], imp[4 * k + 3]};
                    warm_slot(ss, vc[k], ni, ti, A.v, A.w, B.v, B.w);
                    if (ss.flags & 1) st[ss.a] = A;
                    if (ss.flags & 2) st[ss.b] = B;
                }
        }
        if (!frozen) R.vdec[t].assign((size_t)sp.vi * ns, VelDecision{});
        if (tr) tr->wv[t].assign((size_t)sp.vi * ns * 10, (T)0);
        for (int it = 0; it < sp.vi; ++it)
            for (int c = 0; c < ncol; ++c)
                for (int k = co[c]; k < co[c + 1]; ++k) {
                    const SlotStatic ss = slot_static(sl[k]);
                    Body<T> A = st[ss.a], B = st[ss.b];
                    T ni[2] = {imp[4 * k], imp[4 * k + 2]}, ti[2] = {imp[4 * k + 1], imp[4 * k + 3]};
                    if (tr) {
                        T* r = &tr->wv[t][((size_t)it * ns + k) * 10];
                        r[0] = A.v.x; r[1] = A.v.y; r[2] = A.w; r[3] = B.v.x; r[4] = B.v.y; r[5] = B.w;
                        r[6] = ni[0]; r[7] = ti[0]; r[8] = ni[1]; r[9] = ti[1];
                    }
                    VelDecision& d = R.vdec[t][(size_t)it * ns + k];
                    VelDecision dec = frozen ? d : VelDecision{};
                    solve_velocity(ss, vc[k], ni, ti, A.v, A.w, B.v, B.w, dec, frozen);
                    if (!frozen) d = dec;
                    imp[4 * k] = ni[0];
                    imp[4 * k + 1] = ti[0];
                    imp[4 * k + 2] = ni[1];
                    imp[4 * k + 3] = ti[1];
                    if (ss.flags & 1) st[ss.a] = A;
                    if (ss.flags & 2) st[ss.b] = B;
                }
        /* stored impulses (b2_contact_solver_private.rs:585-598): the solved points; a point the
         * reduced block solver left alone keeps what was carried in */
        end_prev.assign(4 * (size_t)ns, (T)0);
        for (int k = 0; k < ns; ++k) {
            for (int j = 0; j < 4; ++j) end_prev[4 * k + j] = raw[4 * k + j];
            for (int j = 0; j < vc[k].vcount; ++j) {
                end_prev[4 * k + 2 * j] = imp[4 * k + 2 * j];
                end_prev[4 * k + 2 * j + 1] = imp[4 * k + 2 * j + 1];
            }
        }
        if (!frozen) R.clamp[t].assign(R.nb, 0);
        if (tr) tr->vel2[t] = st;
        for (int b = 0; b < R.nb; ++b) {
            if (R.bs[b].type == 0) continue;
            unsigned char cl = frozen ? R.clamp[t][b] : 0;
            integrate_position(h, st[b].c, st[b].a, st[b].v, st[b].w, cl, frozen);
            if (!frozen) R.clamp[t][b] = cl;
        }
        if (!frozen) R.pdec[t].assign((size_t)sp.pi * ns * 2, 0);
        if (tr) tr->wp[t].assign((size_t)sp.pi * ns * 6, (T)0);
        for (int it = 0; it < sp.pi; ++it)
            for (int c = 0; c < ncol; ++c)
                for (int k = co[c]; k < co[c + 1]; ++k) {
                    if (it >= pos_iters(sl[k])) continue;
                    const SlotStatic ss = slot_static(sl[k]);
                    Body<T> A = st[ss.a], B = st[ss.b];
                    if (tr) {
                        T* r = &tr->wp[t][((size_t)it * ns + k) * 6];
                        r[0] = A.c.x; r[1] = A.c.y; r[2] = A.a; r[3] = B.c.x; r[4] = B.c.y; r[5] = B.a;
                    }
                    unsigned char* d = &R.pdec[t][((size_t)it * ns + k) * 2];
                    unsigned char dec[2] = {frozen ? d[0] : (unsigned char)0, frozen ? d[1] : (unsigned char)0};
                    const P2<T> lcA = p2((T)sl[k].lc[0], (T)sl[k].lc[1]), lcB = p2((T)sl[k].lc[2], (T)sl[k].lc[3]);
                    solve_position(ss, lcA, lcB, A.c, A.a, B.c, B.a, dec, frozen);
                    if (!frozen) {
                        d[0] = dec[0];
                        d[1] = dec[1];
                    }
                    if (ss.flags & 1) st[ss.a] = A;
                    if (ss.flags & 2) st[ss.b] = B;
                }
    }
    if (!frozen) R.have_dec = true;
}

}  // namespace

extern "C" {

/* col: each step's colour-group offsets (its ncol + 1 ints), concatenated in step order */
void* ora_adj_create(int32_t nb, const float* body_static, int32_t T, const void* steps, const int32_t* col,
                     const void* slots) {
    Ref* R = new Ref;
    R->nb = nb;
    R->bs.resize(nb);
    for (int b = 0; b < nb; ++b) {
        const float* p = body_static + 10 * (size_t)b;
        BodyStatic& s = R->bs[b];
        s.m = p[0];
        s.invm = p[1];
        s.I = p[2];
        s.invI = p[3];
        s.lin_damp = p[4];
        s.ang_damp = p[5];
        s.gscale = p[6];
        s.lcx = p[7];
        s.lcy = p[8];
        s.type = (int)p[9];
    }
    R->T = T;
    R->steps.resize(T);
    std::memcpy(R->steps.data(), steps, (size_t)T * sizeof(HStep));
    R->col.resize(T);
    R->slots.resize(T);
    const HSlot* sp = (const HSlot*)slots;
    size_t off = 0, coff = 0;
    for (int t = 0; t < T; ++t) {
        const int nc = R->steps[t].ncol;
        R->col[t].assign(col + coff, col + coff + nc + 1);
        coff += (size_t)nc + 1;
        R->slots[t].assign(sp + off, sp + off + R->steps[t].nslots);
        off += R->steps[t].nslots;
    }
    return R;
}

void ora_adj_destroy(void* h) { delete (Ref*)h; }

/* state layout: per body c.x, c.y, a, v.x, v.y, w */
int ora_adj_replay_f32(void* h, const float* init, float* out) {
    Ref& R = *(Ref*)h;
    std::vector<Body<float>> st(R.nb);
    for (int b = 0; b < R.nb; ++b) {
        const float* p = init + 6 * (size_t)b;
        st[b].c = p2(p[0], p[1]);
        st[b].a = p[2];
        st[b].v = p2(p[3], p[4]);
        st[b].w = p[5];
    }
    forward<float>(R, false, st, nullptr);
    for (int b = 0; b < R.nb; ++b) {
        float* p = out + 6 * (size_t)b;
        p[0] = st[b].c.x; p[1] = st[b].c.y; p[2] = st[b].a; p[3] = st[b].v.x; p[4] = st[b].v.y; p[5] = st[b].w;
    }
    return (int)(R.carry_mismatch > 0x7fffffff ? 0x7fffffff : R.carry_mismatch);
}

int ora_adj_forward_f64(void* h, const double* init, double* out) {
    Ref& R = *(Ref*)h;
    if (!R.have_dec) return -1;
    std::vector<Body<double>> st(R.nb);
    for (int b = 0; b < R.nb; ++b) {
        const double* p = init + 6 * (size_t)b;
        st[b].c = p2(p[0], p[1]);
        st[b].a = p[2];
        st[b].v = p2(p[3], p[4]);
        st[b].w = p[5];
    }
    forward<double>(R, true, st, nullptr);
    for (int b = 0; b < R.nb; ++b) {
        double* p = out + 6 * (size_t)b;
        p[0] = st[b].c.x; p[1] = st[b].c.y; p[2] = st[b].a; p[3] = st[b].v.x; p[4] = st[b].v.y; p[5] = st[b].w;
    }
    return 0;
}

static int adj_backward(void* h, const double* init, const double* d_final, double* d_init, bool anchored);

int ora_adj_backward_f64(void* h, const double* init, const double* d_final, double* d_init) {
    return adj_backward(h, init, d_final, d_init, false);
}

/* the f64 reverse pass linearised around the f32 replay's trajectory (every step starts from the f32
 * state): isolates the reverse pass's own arithmetic from the f32/f64 trajectories' divergence */
int ora_adj_backward_f64_anchored(void* h, const double* d_final, double* d_init) {
    return adj_backward(h, nullptr, d_final, d_init, true);
}

static int adj_backward(void* h, const double* init, const double* d_final, double* d_init, bool anchored) {
    Ref& R = *(Ref*)h;
    if (!R.have_dec || (anchored && (int)R.anchor_start.size() != R.T) || (!anchored && !init)) return -1;
    typedef double T;
    std::vector<Body<T>> st(R.nb);
    for (int b = 0; b < R.nb; ++b) {
        if (anchored) continue;  /* the forward pass takes every step's start from the f32 replay */
        const double* p = init + 6 * (size_t)b;
        st[b].c = p2(p[0], p[1]);
        st[b].a = p[2];
        st[b].v = p2(p[3], p[4]);
        st[b].w = p[5];
    }
    Trace<T> tr;
    forward<T>(R, true, st, &tr, anchored);
    /* reverse */
    std::vector<Body<T>> g(R.nb);
    for (int b = 0; b < R.nb; ++b) {
        const double* p = d_final + 6 * (size_t)b;
        g[b].c = p2(p[0], p[1]);
        g[b].a = p[2];
        g[b].v = p2(p[3], p[4]);
        g[b].w = p[5];
    }
    std::vector<T> gend_cur(R.T > 0 ? 4 * (size_t)R.steps[R.T - 1].nslots : 0, (T)0), gend_prev;
    for (int t = R.T - 1; t >= 0; --t) {
        const HStep& sp = R.steps[t];
        const std::vector<HSlot>& sl = R.slots[t];
        const std::vector<int>& co = R.col[t];
        const int ns = sp.nslots, ncol = sp.ncol;
        const T h = (T)sp.dt;
        const int nprev = t > 0 ? R.steps[t - 1].nslots : 0;
        gend_prev.assign(4 * (size_t)nprev, (T)0);
        for (int it = sp.pi - 1; it >= 0; --it)
            for (int c = ncol - 1; c >= 0; --c)
                for (int k = co[c]; k < co[c + 1]; ++k) {
                    if (it >= pos_iters(sl[k])) continue;
                    const SlotStatic ss = slot_static(sl[k]);
                    const T* r = &tr.wp[t][((size_t)it * ns + k) * 6];
                    const unsigned char* d = &R.pdec[t][((size_t)it * ns + k) * 2];
                    const P2<T> lcA = p2((T)sl[k].lc[0], (T)sl[k].lc[1]), lcB = p2((T)sl[k].lc[2], (T)sl[k].lc[3]);
                    solve_position_bwd(ss, lcA, lcB, p2(r[0], r[1]), r[2], p2(r[3], r[4]), r[5], d, g[ss.a].c,
                                       g[ss.a].a, g[ss.b].c, g[ss.b].a);
                }
        for (int b = 0; b < R.nb; ++b) {
            if (R.bs[b].type == 0) continue;
            integrate_position_bwd(h, tr.vel2[t][b].v, tr.vel2[t][b].w, R.clamp[t][b], g[b].c, g[b].a, g[b].v,
                                   g[b].w);
        }
        const std::vector<Body<T>>& s0 = tr.start[t];
        const std::vector<Body<T>>& s1 = tr.vel1[t];
        std::vector<VC<T>> vc(ns);
        std::vector<VCGrad<T>> gvc(ns);
        std::vector<T> gimp(4 * (size_t)ns);
        for (int k = 0; k < ns; ++k) {
            const SlotStatic ss = slot_static(sl[k]);
            const P2<T> lcA = p2((T)sl[k].lc[0], (T)sl[k].lc[1]), lcB = p2((T)sl[k].lc[2], (T)sl[k].lc[3]);
            vc[k].vcount = R.vcount[t][k];
            vc[k].bias_on[0] = R.bias[t][2 * k];
            vc[k].bias_on[1] = R.bias[t][2 * k + 1];
            init_slot(ss, s0[ss.a].c, s0[ss.a].a, s0[ss.b].c, s0[ss.b].a, s1[ss.a].v, s1[ss.a].w, s1[ss.b].v,
                      s1[ss.b].w, lcA, lcB, vc[k], true);
            zero(gvc[k]);
            for (int j = 0; j < 4; ++j) gimp[4 * k + j] = gend_cur[4 * k + j];
        }
        for (int it = sp.vi - 1; it >= 0; --it)
            for (int c = ncol - 1; c >= 0; --c)
                for (int k = co[c]; k < co[c + 1]; ++k) {
                    const SlotStatic ss = slot_static(sl[k]);
                    const T* r = &tr.wv[t][((size_t)it * ns + k) * 10];
                    const T ni[2] = {r[6], r[8]}, ti[2] = {r[7], r[9]};
                    T gni[2] = {gimp[4 * k], gimp[4 * k + 2]}, gti[2] = {gimp[4 * k + 1], gimp[4 * k + 3]};
                    solve_velocity_bwd(ss, vc[k], R.vdec[t][(size_t)it * ns + k], ni, ti, p2(r[0], r[1]), r[2],
                                       p2(r[3], r[4]), r[5], gni, gti, g[ss.a].v, g[ss.a].w, g[ss.b].v, g[ss.b].w,
                                       gvc[k]);
                    gimp[4 * k] = gni[0];
                    gimp[4 * k + 1] = gti[0];
                    gimp[4 * k + 2] = gni[1];
                    gimp[4 * k + 3] = gti[1];
                }
        for (int k = 0; k < ns; ++k) {
            const SlotStatic ss = slot_static(sl[k]);
            T gni[2] = {gimp[4 * k], gimp[4 * k + 2]}, gti[2] = {gimp[4 * k + 1], gimp[4 * k + 3]};
            if (sp.warm) {
                const T* i0 = &tr.imp0[t][4 * (size_t)k];
                const T ni0[2] = {i0[0], i0[2]}, ti0[2] = {i0[1], i0[3]};
                warm_slot_bwd(ss, vc[k], ni0, ti0, g[ss.a].v, g[ss.a].w, g[ss.b].v, g[ss.b].w, gni, gti, gvc[k]);
            }
            for (int j = 0; j < ss.count; ++j) {
                T gn, gt;
                if (j < vc[k].vcount) {
                    gn = sp.warm ? (T)sp.dt_ratio * gni[j] : (T)0;
                    gt = sp.warm ? (T)sp.dt_ratio * gti[j] : (T)0;
                } else {
                    gn = gend_cur[4 * k + 2 * j];
                    gt = gend_cur[4 * k + 2 * j + 1];
                }
                const int cj = ss.carry[j];
                if (cj >= 0 && t > 0) {
                    gend_prev[2 * (size_t)cj] += gn;
                    gend_prev[2 * (size_t)cj + 1] += gt;
                }
            }
        }
        for (int c = ncol - 1; c >= 0; --c)
            for (int k = co[c]; k < co[c + 1]; ++k) {
                const SlotStatic ss = slot_static(sl[k]);
                const P2<T> lcA = p2((T)sl[k].lc[0], (T)sl[k].lc[1]), lcB = p2((T)sl[k].lc[2], (T)sl[k].lc[3]);
                init_slot_bwd(ss, s0[ss.a].c, s0[ss.a].a, s0[ss.b].c, s0[ss.b].a, s1[ss.a].v, s1[ss.a].w, s1[ss.b].v,
                              s1[ss.b].w, lcA, lcB, vc[k], gvc[k], g[ss.a].c, g[ss.a].a, g[ss.b].c, g[ss.b].a,
                              g[ss.a].v, g[ss.a].w, g[ss.b].v, g[ss.b].w);
            }
        for (int b = 0; b < R.nb; ++b)
            if (R.bs[b].type == 2) integrate_velocity_bwd(R.bs[b], h, g[b].v, g[b].w);
        gend_cur.swap(gend_prev);
    }
    for (int b = 0; b < R.nb; ++b) {
        double* p = d_init + 6 * (size_t)b;
        p[0] = g[b].c.x; p[1] = g[b].c.y; p[2] = g[b].a; p[3] = g[b].v.x; p[4] = g[b].v.y; p[5] = g[b].w;
    }
    return 0;
}

}  // extern "C"
