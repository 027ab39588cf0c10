/*
 * k_solver.cu — islands, constraint colouring and the contact solver of a step.
 *
 * Reference: B2world::solve (src/private/dynamics/b2_world.rs:356-531), B2island::solve
 * (src/private/dynamics/b2_island_private.rs:129-328) and B2contactSolver
 * (src/private/dynamics/b2_contact_solver_private.rs:20-730).
 *
 * GPU formulation
 *   islands     lock-free union-find over touching contacts whose bodies are both
 *               non-static (the reference's DFS does not cross static bodies); the
 *               root is the smallest body index, so labels are deterministic. An
 *               island is solved if any member is awake; its members are woken.
 *   constraints the touching, enabled, non-sensor contacts of solved islands, compacted
 *               in contact-table order by a scan.
 *   colouring   constraints that persist from the previous colouring keep their colour;
 *               the new ones are coloured in rounds of: every uncoloured constraint whose
 *               hashed priority is the minimum at both of its dynamic bodies takes the
 *               lowest colour unused at either body (first fit over 64 colours; past that,
 *               one colour per round). Constraints of one colour share no dynamic body, so
 *               each colour is solved in parallel with results identical to any sequential
 *               order.
 *   solver      one persistent cooperative kernel: integrate velocities, initialise
 *               constraints, warm start, velocity iterations, store impulses, integrate
 *               positions, position iterations with the per-island early exit, write
 *               back transforms, sleep, synchronise fixtures (fat AABB + moved flag).
 *               Colour sweeps are separated by a grid barrier whose wait is bounded:
 *               on timeout it sets ST_BARRIER_TIMEOUT and the kernel returns.
 * The host reference solved in the GPU's colour order (the oracle's ordering hook)
 * gives bit-identical bodies, because each operation is the same IEEE f32 operation.
 */
#include "b2g_internal.h"
#include "b2g_sync.cuh"

namespace b2g {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ bool is_dynamic(uint32_t flags) { return (flags & BF_TYPE_MASK) == BODY_DYNAMIC; }
__device__ __forceinline__ bool is_static(uint32_t flags) { return (flags & BF_TYPE_MASK) == BODY_STATIC; }


/* ---------------- islands ---------------- */
__device__ __forceinline__ int uf_find(int* parent, int x) {
    int p = parent[x];
    while (p != x) {
        const int gp = parent[p];
        if (gp != p) parent[x] = gp;  /* path halving; any stale value is still an ancestor */
        x = p;
        p = gp;
    }
    return x;
}

__device__ __forceinline__ void uf_union(int* parent, int a, int b) {
    for (int guard = 0; guard < 1 << 20; ++guard) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        const int hi = a > b ? a : b, lo = a > b ? b : a;
        if (atomicCAS(&parent[hi], hi, lo) == hi) return;
    }
}

__global__ void k_island_init(DevWorld w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x) {
        w.b_island[b] = b;
        w.isl_minsep[w.body_cap + b] = 0u;  /* "island has an awake member" */
        w.b_flags[b] &= ~BF_ISLAND;
    }
}

__device__ __forceinline__ bool contact_is_constraint(uint32_t cf) {
    return (cf & (CF_TOUCHING | CF_ENABLED | CF_DEAD | CF_SENSOR)) == (CF_TOUCHING | CF_ENABLED);
}

__global__ void k_island_union(DevWorld w) {
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!contact_is_constraint(w.c.flags[i])) continue;
        const int2 bd = w.c.body[i];
        if (is_static(w.b_flags[bd.x]) || is_static(w.b_flags[bd.y])) continue;
        uf_union(w.b_island, bd.x, bd.y);
    }
}

__global__ void k_island_compress(DevWorld w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x) {
        const int r = uf_find(w.b_island, b);
        const uint32_t f = w.b_flags[b];
        if ((f & BF_AWAKE) && (f & BF_ENABLED) && !is_static(f)) atomicOr(&w.isl_minsep[w.body_cap + r], 1u);
    }
}

__global__ void k_island_mark(DevWorld w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x) {
        int r = w.b_island[b];
        r = w.b_island[r];  /* compress left every body at most one hop from its root */
        while (w.b_island[r] != r) r = w.b_island[r];
        w.b_island[b] = r;
        const uint32_t f = w.b_flags[b];
        if (!is_static(f) && (f & BF_ENABLED) && w.isl_minsep[w.body_cap + r]) w.b_flags[b] = f | BF_AWAKE | BF_ISLAND;
    }
}

/* flag[i] = 1 if contact i is a constraint of a solved island */
__global__ void k_cons_flags(DevWorld w, uint32_t* flag) {
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t sel = 0;
        if (contact_is_constraint(w.c.flags[i])) {
            const int2 bd = w.c.body[i];
            const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
            sel = ((fa & BF_ISLAND) || (fb & BF_ISLAND)) ? 1u : 0u;
        }
        flag[i] = sel;
    }
}

__global__ void k_cons_scatter(DevWorld w, const uint32_t* flag, const uint32_t* pos) {
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        const int k = (int)pos[i];
        if (k >= w.cons_cap) {
            atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_CONTACT_OVERFLOW);
            continue;
        }
        const int2 bd = w.c.body[i];
        const int b = is_static(w.b_flags[bd.x]) ? bd.y : bd.x;
        w.cons_contact[k] = i;
        w.cons_island[k] = w.b_island[b];
    }
}

__global__ void k_cons_clamp(DevWorld w) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && w.cnt[CNT_CONS] > w.cons_cap) w.cnt[CNT_CONS] = w.cons_cap;
}

/* ---------------- colouring (cooperative) ---------------- */
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

/* Colouring. A constraint that was also a constraint of the previous colouring keeps its
 * first-fit colour (stored in its contact with that colouring's stamp): the previous colours were
 * a proper colouring of the previous constraints, so any subset of them still is. Only the new
 * constraints are coloured, by Jones-Plassmann rounds (hash priorities; a local minimum at both
 * of its dynamic bodies takes the lowest colour free at both), so a step whose contacts persist
 * needs one or two rounds instead of one per colour. */
__global__ void __launch_bounds__(kBlock) k_colour(DevWorld w) {
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    const int n = w.cnt[CNT_CONS];
    const unsigned long long kNone = ~0ull;
    const uint32_t stamp = (uint32_t)w.cnt[CNT_COLOURINGS] & 0x3ffffffu;  /* the previous colouring's */
    /* offers are double-buffered by round parity: round r offers into buffer r & 1, and the
     * entries of buffer (r - 1) & 1 are reset during round r, so a round needs two barriers */
    for (int b = gtid; b < w.n_bodies; b += gsize) {
        w.b_cmin[b] = kNone;
        w.b_cmin[w.body_cap + b] = kNone;
        w.b_cmask[b] = 0ull;
    }
    /* every 16th colouring starts afresh, so kept colours do not stay fragmented after the
     * contact graph has changed (a fresh colouring of a settled stack needs fewer colours) */
    const bool keep = stamp != 0u && (stamp & 15u) != 0u;
    for (int k = gtid; k < n; k += gsize) {
        const uint32_t kept = w.c.mids[w.cons_contact[k]].w;
        w.cons_colour[k] = (keep && (kept >> 6) == stamp) ? (int)(kept & 63u) : -1;
    }
    for (int c = gtid; c < kMaxColours; c += gsize) w.col_hist[c] = 0;
    if (!grid_barrier(w)) return;
    /* the kept colours are taken at their bodies */
    for (int k = gtid; k < n; k += gsize) {
        const int c = w.cons_colour[k];
        if (c < 0) continue;
        const int2 bd = w.c.body[w.cons_contact[k]];
        const unsigned long long bit = 1ull << c;
        if (is_dynamic(w.b_flags[bd.x])) atomicOr(&w.b_cmask[bd.x], bit);
        if (is_dynamic(w.b_flags[bd.y])) atomicOr(&w.b_cmask[bd.y], bit);
    }
    if (gtid == 0) {
        /* two "still uncoloured" counters alternate by round parity: round r counts into
         * [r & 1] and reads the previous round's result from [(r + 1) & 1] */
        w.cnt[CNT_UNCOLOURED] = 0;
        w.cnt[CNT_UNCOLOURED + 1] = n;
        w.cnt[CNT_ROUNDS] = 0;
    }
    if (!grid_barrier(w)) return;
    int round = 0;
    for (;;) {
        const int remaining = ((volatile int*)w.cnt)[CNT_UNCOLOURED + ((round + 1) & 1)];
        if (remaining <= 0) break;
        if (round >= kMaxColours - kFirstFitColours) {
            /* cannot happen for rounds bounded by the maximum body degree; keep the kernel finite */
            for (int k = gtid; k < n; k += gsize)
                if (w.cons_colour[k] < 0) w.cons_colour[k] = kMaxColours - 1;
            if (gtid == 0) atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_COLOUR_OVERFLOW);
            break;
        }
        unsigned long long* offer = w.b_cmin + (size_t)(round & 1) * w.body_cap;
        unsigned long long* stale = w.b_cmin + (size_t)((round + 1) & 1) * w.body_cap;
        /* A: each uncoloured constraint offers its priority to its dynamic bodies */
        for (int k = gtid; k < n; k += gsize) {
            const int2 bd = w.c.body[w.cons_contact[k]];
            if (round > 0) {
                stale[bd.x] = kNone;
                stale[bd.y] = kNone;
            }
            if (w.cons_colour[k] >= 0) continue;
            const unsigned long long key = ((unsigned long long)hash32((uint32_t)k) << 32) | (uint32_t)k;
            if (is_dynamic(w.b_flags[bd.x])) atomicMin(&offer[bd.x], key);
            if (is_dynamic(w.b_flags[bd.y])) atomicMin(&offer[bd.y], key);
        }
        if (gtid == 0) w.cnt[CNT_UNCOLOURED + (round & 1)] = 0;
        if (!grid_barrier(w)) return;
        /* B: local minima take the lowest colour free at both bodies */
        for (int k = gtid; k < n; k += gsize) {
            if (w.cons_colour[k] >= 0) continue;
            const int2 bd = w.c.body[w.cons_contact[k]];
            const unsigned long long key = ((unsigned long long)hash32((uint32_t)k) << 32) | (uint32_t)k;
            const bool da = is_dynamic(w.b_flags[bd.x]), db = is_dynamic(w.b_flags[bd.y]);
            const bool winA = !da || offer[bd.x] == key;
            const bool winB = !db || offer[bd.y] == key;
            if (winA && winB) {
                const unsigned long long used = (da ? w.b_cmask[bd.x] : 0ull) | (db ? w.b_cmask[bd.y] : 0ull);
                int colour;
                if (~used != 0ull) {
                    colour = __ffsll((long long)~used) - 1;
                    const unsigned long long bit = 1ull << colour;
                    if (da) w.b_cmask[bd.x] |= bit;
                    if (db) w.b_cmask[bd.y] |= bit;
                } else {
                    colour = kFirstFitColours + round;
                    if (colour >= kMaxColours) {
                        colour = kMaxColours - 1;
                        atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_COLOUR_OVERFLOW);
                    }
                }
                w.cons_colour[k] = colour;
            } else {
                atomicAdd(&w.cnt[CNT_UNCOLOURED + (round & 1)], 1);
            }
        }
        ++round;
        if (!grid_barrier(w)) return;
    }
    if (gtid == 0) w.cnt[CNT_ROUNDS] = round;
    /* histogram, dense colour offsets, scatter into slots */
    for (int k = gtid; k < n; k += gsize) atomicAdd(&w.col_hist[w.cons_colour[k]], 1);
    if (!grid_barrier(w)) return;
    if (blockIdx.x == 0) {
        __shared__ int s_cnt[kMaxColours];
        __shared__ int s_dense[kMaxColours];
        for (int c = threadIdx.x; c < kMaxColours; c += blockDim.x) s_cnt[c] = w.col_hist[c];
        __syncthreads();
        if (threadIdx.x == 0) {
            int base = 0, dense = 0;
            for (int c = 0; c < kMaxColours; ++c) {
                if (s_cnt[c] == 0) {
                    s_dense[c] = -1;
                    continue;
                }
                w.col_off[dense] = base;
                s_dense[c] = base;  /* running cursor start */
                base += s_cnt[c];
                ++dense;
            }
            w.col_off[dense] = base;
            w.cnt[CNT_COLOURS] = dense;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < kMaxColours; c += blockDim.x) w.col_hist[c] = s_dense[c];  /* cursor */
    }
    if (!grid_barrier(w)) return;
    const uint32_t next = (stamp + 1u) & 0x3ffffffu;
    for (int k = gtid; k < n; k += gsize) {
        const int c = w.cons_colour[k];
        const int ci = w.cons_contact[k];
        const int slot = atomicAdd(&w.col_hist[c], 1);
        /* keep first-fit colours for the next colouring (the per-round overflow colours are not
         * kept: a later round could hand the same one to a neighbour) */
        w.c.mids[ci].w = (c < kFirstFitColours && next != 0u) ? ((next << 6) | (uint32_t)c) : 0u;
        if (slot < 0 || slot >= n) continue;  /* cannot happen with consistent offsets */
        w.s_contact[slot] = ci;
        w.s_cons[slot] = k;
    }
    if (gtid == 0) w.cnt[CNT_COLOURINGS] = (int)next;
}

/* ---------------- solver (cooperative) ---------------- */
__device__ __forceinline__ V2 v2of(float x, float y) { return mk(x, y); }

/* B2contactSolver::new + initialize_velocity_constraints for one slot */
__device__ void init_slot(const DevWorld& w, const StepParams& sp, int k) {
    const int ci = w.s_contact[k];
    const int2 fx = w.c.fix[ci];
    const int2 bd = w.c.body[ci];
    const float4 mat = w.c.mat[ci];
    const float4 geo = w.c.mgeo[ci];
    const float4 pts = w.c.mpts[ci];
    const float4 imp = w.c.mimp[ci];
    const uint4 ids = w.c.mids[ci];
    const int mtype = (int)(ids.z & 0xffu);
    const int count = (int)((ids.z >> 8) & 0xffu);
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float mA = massA.y, iA = massA.w, mB = massB.y, iB = massB.w;
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float4 pA = w.b_pos[bd.x], pB = w.b_pos[bd.y];
    const float4 vA4 = w.b_vel[bd.x], vB4 = w.b_vel[bd.y];
    const float rA = w.f_shape[fx.x].radius, rB = w.f_shape[fx.y].radius;
    const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];

    float ni0 = 0.0f, ti0 = 0.0f, ni1 = 0.0f, ti1 = 0.0f;
    if (sp.warm) {
        ni0 = sp.dt_ratio * imp.x;
        ti0 = sp.dt_ratio * imp.y;
        if (count > 1) {
            ni1 = sp.dt_ratio * imp.z;
            ti1 = sp.dt_ratio * imp.w;
        }
    }
    const V2 cA = v2of(pA.x, pA.y), cB = v2of(pB.x, pB.y);
    const V2 vA = v2of(vA4.x, vA4.y), vB = v2of(vB4.x, vB4.y);
    const float wA = vA4.z, wB = vB4.z;
    Xf xfA, xfB;
    xfA.q = rot(pA.z);
    xfB.q = rot(pB.z);
    xfA.p = sub(cA, mul(xfA.q, mk(lcA.x, lcA.y)));
    xfB.p = sub(cB, mul(xfB.q, mk(lcB.x, lcB.y)));
    /* b2_world_manifold_initialize, private/collision/b2_collision.rs:7-68 */
    V2 normal = mk(1.0f, 0.0f);
    V2 wp[2] = {mk(0.0f, 0.0f), mk(0.0f, 0.0f)};
    const V2 ln = mk(geo.x, geo.y), lpt = mk(geo.z, geo.w);
    const V2 lp[2] = {mk(pts.x, pts.y), mk(pts.z, pts.w)};
    if (mtype == MANIFOLD_CIRCLES) {
        V2 pa = mul(xfA, lpt);
        V2 pb = mul(xfB, lp[0]);
        if (dist_sq(pa, pb) > kEpsilon * kEpsilon) {
            normal = sub(pb, pa);
            normalize(normal);
        }
        V2 ca = add(pa, scale(rA, normal));
        V2 cb = sub(pb, scale(rB, normal));
        wp[0] = scale(0.5f, add(ca, cb));
    } else if (mtype == MANIFOLD_FACE_A) {
        normal = mul(xfA.q, ln);
        V2 plane = mul(xfA, lpt);
        for (int j = 0; j < count; ++j) {
            V2 clip = mul(xfB, lp[j]);
            V2 ca = add(clip, scale(rA - dot(sub(clip, plane), normal), normal));
            V2 cb = sub(clip, scale(rB, normal));
            wp[j] = scale(0.5f, add(ca, cb));
        }
    } else {
        normal = mul(xfB.q, ln);
        V2 plane = mul(xfB, lpt);
        for (int j = 0; j < count; ++j) {
            V2 clip = mul(xfA, lp[j]);
            V2 cb = add(clip, scale(rB - dot(sub(clip, plane), normal), normal));
            V2 ca = sub(clip, scale(rA, normal));
            wp[j] = scale(0.5f, add(ca, cb));
        }
        normal = neg(normal);
    }
    V2 ra[2], rb[2];
    float nm[2] = {0.0f, 0.0f}, tm[2] = {0.0f, 0.0f}, bias[2] = {0.0f, 0.0f};
    const V2 tangent = cross_vs(normal, 1.0f);
    for (int j = 0; j < 2; ++j) {
        ra[j] = mk(0.0f, 0.0f);
        rb[j] = mk(0.0f, 0.0f);
    }
    for (int j = 0; j < count; ++j) {
        ra[j] = sub(wp[j], cA);
        rb[j] = sub(wp[j], cB);
        float rnA = cross(ra[j], normal);
        float rnB = cross(rb[j], normal);
        float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        nm[j] = kNormal > 0.0f ? fdiv(1.0f, kNormal) : 0.0f;
        float rtA = cross(ra[j], tangent);
        float rtB = cross(rb[j], tangent);
        float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
        tm[j] = kTangent > 0.0f ? fdiv(1.0f, kTangent) : 0.0f;
        float vRel = dot(normal, sub(sub(add(vB, cross_sv(wB, rb[j])), vA), cross_sv(wA, ra[j])));
        if (vRel < -mat.z) bias[j] = -mat.y * vRel;
    }
    int vcount = count;
    float k11 = 0.0f, k12 = 0.0f, k22 = 0.0f, na = 0.0f, nb = 0.0f, nd = 0.0f;
    if (count == 2) {
        float rn1A = cross(ra[0], normal);
        float rn1B = cross(rb[0], normal);
        float rn2A = cross(ra[1], normal);
        float rn2B = cross(rb[1], normal);
        k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
        k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
        k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
        const float kMaxConditionNumber = 1000.0f;
        if (k11 * k11 < kMaxConditionNumber * (k11 * k22 - k12 * k12)) {
            /* B2Mat22::get_inverse of [[k11, k12], [k12, k22]] */
            float det = k11 * k22 - k12 * k12;
            if (det != 0.0f) det = fdiv(1.0f, det);
            na = det * k22;      /* ex.x */
            /* ex.y = -det * k12 equals ey.x (K is symmetric) */
            nb = -det * k12;     /* ey.x */
            nd = det * k11;      /* ey.y */
        } else {
            vcount = 1;
            k11 = k12 = k22 = 0.0f;
        }
    }
    const int flagsAB = (is_dynamic(fa) ? 1 : 0) | (is_dynamic(fb) ? 2 : 0);
    w.vc_idx[k] = make_int4(bd.x, bd.y, vcount, flagsAB);
    w.vc_inv[k] = make_float4(mA, mB, iA, iB);
    w.vc_nf[k] = make_float4(normal.x, normal.y, mat.x, mat.w);
    w.vc_r0[k] = make_float4(ra[0].x, ra[0].y, rb[0].x, rb[0].y);
    w.vc_r1[k] = make_float4(ra[1].x, ra[1].y, rb[1].x, rb[1].y);
    /* the inverse's off-diagonal (nb == nc) and ey.y ride in the spare lanes */
    w.vc_m0[k] = make_float4(nm[0], tm[0], bias[0], nb);
    w.vc_m1[k] = make_float4(nm[1], tm[1], bias[1], nd);
    w.vc_imp[k] = make_float4(ni0, ti0, ni1, ti1);
    /* K = [[k11, k12], [k12, k22]] and its inverse ([[na, nb], [nc, nd]], nb == nc) */
    w.vc_k[k] = make_float4(k11, k12, k22, na);
    w.pc_lp[k] = make_float4(lp[0].x, lp[0].y, lp[1].x, lp[1].y);
    w.pc_geo[k] = make_float4(ln.x, ln.y, lpt.x, lpt.y);
    w.pc_lc[k] = make_float4(lcA.x, lcA.y, lcB.x, lcB.y);
    w.pc_inv[k] = make_float4(mA, mB, iA, iB);
    w.pc_meta[k] = make_float4(rA, rB, __int_as_float(mtype), __int_as_float(count));
    w.vc_island[k] = w.cons_island[w.s_cons[k]];
    w.s_fix[k] = fx;
}

__device__ __forceinline__ void warm_slot(const DevWorld& w, int k) {
    const int4 idx = w.vc_idx[k];
    const float4 inv = w.vc_inv[k];
    const float4 nf = w.vc_nf[k];
    const float4 imp = w.vc_imp[k];
    float4 va = w.b_vel[idx.x], vb = w.b_vel[idx.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const V2 normal = mk(nf.x, nf.y);
    const V2 tangent = cross_vs(normal, 1.0f);
    const float4 r[2] = {w.vc_r0[k], w.vc_r1[k]};
    const float ni[2] = {imp.x, imp.z}, ti[2] = {imp.y, imp.w};
    for (int j = 0; j < idx.z; ++j) {
        const V2 rA = mk(r[j].x, r[j].y), rB = mk(r[j].z, r[j].w);
        const V2 P = add(scale(ni[j], normal), scale(ti[j], tangent));
        wA -= inv.z * cross(rA, P);
        vA = sub(vA, scale(inv.x, P));
        wB += inv.w * cross(rB, P);
        vB = add(vB, scale(inv.y, P));
    }
    if (idx.w & 1) w.b_vel[idx.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (idx.w & 2) w.b_vel[idx.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ __forceinline__ void solve_velocity_slot(const DevWorld& w, int k) {
    const int4 idx = w.vc_idx[k];
    const float4 inv = w.vc_inv[k];
    const float4 nf = w.vc_nf[k];
    float4 imp = w.vc_imp[k];
    const float4 r0 = w.vc_r0[k], r1 = w.vc_r1[k];
    const float4 m0 = w.vc_m0[k], m1 = w.vc_m1[k];
    const float mA = inv.x, mB = inv.y, iA = inv.z, iB = inv.w;
    float4 va = w.b_vel[idx.x], vb = w.b_vel[idx.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const V2 normal = mk(nf.x, nf.y);
    const V2 tangent = cross_vs(normal, 1.0f);
    const float friction = nf.z;
    const V2 rA0 = mk(r0.x, r0.y), rB0 = mk(r0.z, r0.w), rA1 = mk(r1.x, r1.y), rB1 = mk(r1.z, r1.w);
    /* friction first (b2_contact_solver_private.rs:295-323) */
    {
        V2 dv = sub(sub(add(vB, cross_sv(wB, rB0)), vA), cross_sv(wA, rA0));
        float vt = dot(dv, tangent) - nf.w;
        float lambda = m0.y * (-vt);
        float maxFriction = friction * imp.x;
        float newImpulse = fclampr(imp.y + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - imp.y;
        imp.y = newImpulse;
        V2 P = scale(lambda, tangent);
        vA = sub(vA, scale(mA, P));
        wA -= iA * cross(rA0, P);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB0, P);
    }
    if (idx.z == 2) {
        V2 dv = sub(sub(add(vB, cross_sv(wB, rB1)), vA), cross_sv(wA, rA1));
        float vt = dot(dv, tangent) - nf.w;
        float lambda = m1.y * (-vt);
        float maxFriction = friction * imp.z;
        float newImpulse = fclampr(imp.w + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - imp.w;
        imp.w = newImpulse;
        V2 P = scale(lambda, tangent);
        vA = sub(vA, scale(mA, P));
        wA -= iA * cross(rA1, P);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB1, P);
    }
    if (idx.z == 1) {
        V2 dv = sub(sub(add(vB, cross_sv(wB, rB0)), vA), cross_sv(wA, rA0));
        float vn = dot(dv, normal);
        float lambda = -m0.x * (vn - m0.z);
        float newImpulse = fmaxr(imp.x + lambda, 0.0f);
        lambda = newImpulse - imp.x;
        imp.x = newImpulse;
        V2 P = scale(lambda, normal);
        vA = sub(vA, scale(mA, P));
        wA -= iA * cross(rA0, P);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB0, P);
    } else {
        /* 2-point block LCP, b2_contact_solver_private.rs:380-575 */
        const float4 K = w.vc_k[k];
        const float k11 = K.x, k12 = K.y, k22 = K.z;
        const float na = K.w, nbc = m0.w, nd = m1.w;
        const V2 a = mk(imp.x, imp.z);
        V2 dv1 = sub(sub(add(vB, cross_sv(wB, rB0)), vA), cross_sv(wA, rA0));
        V2 dv2 = sub(sub(add(vB, cross_sv(wB, rB1)), vA), cross_sv(wA, rA1));
        float vn1 = dot(dv1, normal);
        float vn2 = dot(dv2, normal);
        V2 b = mk(vn1 - m0.z, vn2 - m1.z);
        /* b -= K * a */
        b = sub(b, mk(k11 * a.x + k12 * a.y, k12 * a.x + k22 * a.y));
        V2 x;
        bool solved = false;
        /* case 1: x = -inv(K) b */
        x = neg(mk(na * b.x + nbc * b.y, nbc * b.x + nd * b.y));
        if (x.x >= 0.0f && x.y >= 0.0f) solved = true;
        if (!solved) {
            x.x = -m0.x * b.x;
            x.y = 0.0f;
            vn2 = k12 * x.x + b.y;
            if (x.x >= 0.0f && vn2 >= 0.0f) solved = true;
        }
        if (!solved) {
            x.x = 0.0f;
            x.y = -m1.x * b.y;
            vn1 = k12 * x.y + b.x;
            if (x.y >= 0.0f && vn1 >= 0.0f) solved = true;
        }
        if (!solved) {
            x.x = 0.0f;
            x.y = 0.0f;
            vn1 = b.x;
            vn2 = b.y;
            if (vn1 >= 0.0f && vn2 >= 0.0f) solved = true;
        }
        if (solved) {
            V2 d = sub(x, a);
            V2 P1 = scale(d.x, normal);
            V2 P2 = scale(d.y, normal);
            vA = sub(vA, scale(mA, add(P1, P2)));
            wA -= iA * (cross(rA0, P1) + cross(rA1, P2));
            vB = add(vB, scale(mB, add(P1, P2)));
            wB += iB * (cross(rB0, P1) + cross(rB1, P2));
            imp.x = x.x;
            imp.z = x.y;
        }
    }
    w.vc_imp[k] = imp;
    if (idx.w & 1) w.b_vel[idx.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (idx.w & 2) w.b_vel[idx.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_position_constraints for one slot; returns this slot's min separation (<= 0) */
__device__ __forceinline__ float solve_position_slot(const DevWorld& w, int k) {
    const int4 idx = w.vc_idx[k];
    const float4 lp = w.pc_lp[k], geo = w.pc_geo[k], lc = w.pc_lc[k], inv = w.pc_inv[k], meta = w.pc_meta[k];
    const float mA = inv.x, mB = inv.y, iA = inv.z, iB = inv.w;
    const V2 lcA = mk(lc.x, lc.y), lcB = mk(lc.z, lc.w);
    const int mtype = __float_as_int(meta.z);
    const int count = __float_as_int(meta.w);
    const float rA = meta.x, rB = meta.y;
    const V2 ln = mk(geo.x, geo.y), lpt = mk(geo.z, geo.w);
    const V2 lps[2] = {mk(lp.x, lp.y), mk(lp.z, lp.w)};
    float4 pa = w.b_pos[idx.x], pb = w.b_pos[idx.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    float minSep = 0.0f;
    for (int j = 0; j < count; ++j) {
        Xf xfA, xfB;
        xfA.q = rot(aA);
        xfB.q = rot(aB);
        xfA.p = sub(cA, mul(xfA.q, lcA));
        xfB.p = sub(cB, mul(xfB.q, lcB));
        V2 normal, point;
        float separation;
        if (mtype == MANIFOLD_CIRCLES) {
            V2 pA = mul(xfA, lpt);
            V2 pB = mul(xfB, lps[0]);
            normal = sub(pB, pA);
            normalize(normal);
            point = scale(0.5f, add(pA, pB));
            separation = dot(sub(pB, pA), normal) - rA - rB;
        } else if (mtype == MANIFOLD_FACE_A) {
            normal = mul(xfA.q, ln);
            V2 plane = mul(xfA, lpt);
            V2 clip = mul(xfB, lps[j]);
            separation = dot(sub(clip, plane), normal) - rA - rB;
            point = clip;
        } else {
            normal = mul(xfB.q, ln);
            V2 plane = mul(xfB, lpt);
            V2 clip = mul(xfA, lps[j]);
            separation = dot(sub(clip, plane), normal) - rA - rB;
            point = clip;
            normal = neg(normal);
        }
        V2 ra = sub(point, cA);
        V2 rb = sub(point, cB);
        minSep = fminr(minSep, separation);
        float C = fclampr(kBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
        float rnA = cross(ra, normal);
        float rnB = cross(rb, normal);
        float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        float impulse = K > 0.0f ? fdiv(-C, K) : 0.0f;
        V2 P = scale(impulse, normal);
        cA = sub(cA, scale(mA, P));
        aA -= iA * cross(ra, P);
        cB = add(cB, scale(mB, P));
        aB += iB * cross(rb, P);
    }
    if (idx.w & 1) w.b_pos[idx.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (idx.w & 2) w.b_pos[idx.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return minSep;
}

/* B2dynamicTree::move_proxy, private/collision/b2_dynamic_tree.rs:109-168 (fat AABB rule only) */
__device__ __forceinline__ void move_proxy(const DevWorld& w, int f, const AABB& aabb, V2 disp) {
    const V2 r = mk(kAabbExtension, kAabbExtension);
    AABB fat;
    fat.lo = sub(aabb.lo, r);
    fat.hi = add(aabb.hi, r);
    const V2 d = scale(kAabbMultiplier, disp);
    if (d.x < 0.0f) fat.lo.x += d.x; else fat.hi.x += d.x;
    if (d.y < 0.0f) fat.lo.y += d.y; else fat.hi.y += d.y;
    const float4 t = w.f_fat[f];
    AABB tree;
    tree.lo = mk(t.x, t.y);
    tree.hi = mk(t.z, t.w);
    if (contains(tree, aabb)) {
        AABB huge;
        huge.lo = sub(fat.lo, scale(4.0f, r));
        huge.hi = add(fat.hi, scale(4.0f, r));
        if (contains(huge, tree)) return;
    }
    w.f_fat[f] = make_float4(fat.lo.x, fat.lo.y, fat.hi.x, fat.hi.y);
    w.f_moved[f] = 1;
}

__device__ __forceinline__ void sync_fixture(const DevWorld& w, int f, const Xf& xf1, const Xf& xf2) {
    const ShapeRec s = w.f_shape[f];
    AABB a1, a2;
    shape_aabb(s, xf1, a1);
    shape_aabb(s, xf2, a2);
    const AABB swept = combine(a1, a2);
    const V2 disp = sub(center(a2), center(a1));
    move_proxy(w, f, swept, disp);
}

__global__ void __launch_bounds__(kBlock) k_solve(DevWorld w, StepParams sp) {
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    const int nb = w.n_bodies;
    const int ncons = w.cnt[CNT_CONS];
    const int ncol = w.cnt[CNT_COLOURS];
    const float h = sp.dt;
    /* phase 0: integrate velocities (b2_island_private.rs:136-170) */
    for (int b = gtid; b < nb; b += gsize) {
        const uint32_t f = w.b_flags[b];
        if (!(f & BF_ISLAND)) continue;
        const float4 p = w.b_pos[b];
        w.b_pos0[b] = p;
        if (is_dynamic(f)) {
            float4 v = w.b_vel[b];
            const float4 m = w.b_mass[b];
            const float4 fo = w.b_force[b];
            const float4 d = w.b_damp[b];
            const float s = h * m.y;
            const float gm = d.z * m.x;
            const float gx = gm * sp.gx + fo.x;
            const float gy = gm * sp.gy + fo.y;
            v.x += s * gx;
            v.y += s * gy;
            v.z += h * m.w * fo.z;
            const float ld = fdiv(1.0f, 1.0f + h * d.x);
            const float ad = fdiv(1.0f, 1.0f + h * d.y);
            v.x *= ld;
            v.y *= ld;
            v.z *= ad;
            w.b_vel[b] = v;
        }
    }
    if (!grid_barrier(w)) return;
    /* phase 1: constraint initialisation */
    for (int k = gtid; k < ncons; k += gsize) init_slot(w, sp, k);
    if (!grid_barrier(w)) return;
    /* phase 2: warm start, colour by colour */
    if (sp.warm) {
        for (int c = 0; c < ncol; ++c) {
            const int beg = w.col_off[c], end = w.col_off[c + 1];
            for (int k = beg + gtid; k < end; k += gsize) warm_slot(w, k);
            if (!grid_barrier(w)) return;
        }
    }
    /* phase 3: velocity iterations */
    for (int it = 0; it < sp.vi; ++it) {
        for (int c = 0; c < ncol; ++c) {
            const int beg = w.col_off[c], end = w.col_off[c + 1];
            for (int k = beg + gtid; k < end; k += gsize) solve_velocity_slot(w, k);
            if (!grid_barrier(w)) return;
        }
    }
    /* phase 4: store impulses (:585-598) and integrate positions (:222-252) */
    for (int k = gtid; k < ncons; k += gsize) {
        const int ci = w.s_contact[k];
        const int4 idx = w.vc_idx[k];
        const float4 imp = w.vc_imp[k];
        float4 m = w.c.mimp[ci];
        m.x = imp.x;
        m.y = imp.y;
        if (idx.z > 1) {
            m.z = imp.z;
            m.w = imp.w;
        }
        w.c.mimp[ci] = m;
    }
    for (int b = gtid; b < nb; b += gsize) {
        const uint32_t f = w.b_flags[b];
        if (!(f & BF_ISLAND)) continue;
        float4 p = w.b_pos[b];
        float4 v = w.b_vel[b];
        V2 vv = mk(v.x, v.y);
        float wv = v.z;
        V2 translation = scale(h, vv);
        if (dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = fdiv(kMaxTranslation, length(translation));
            vv.x *= ratio;
            vv.y *= ratio;
        }
        float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = fdiv(kMaxRotation, fabsr(rotation));
            wv *= ratio;
        }
        p.x += h * vv.x;
        p.y += h * vv.y;
        p.z += h * wv;
        w.b_pos[b] = p;
        w.b_vel[b] = make_float4(vv.x, vv.y, wv, v.w);
        for (int j = 0; j < sp.pi; ++j) w.isl_minsep[(size_t)j * w.body_cap + b] = 0u;
    }
    if (!grid_barrier(w)) return;
    /* phase 5: position iterations with the per-island early exit (:257-274).
     * Iteration j accumulates max(-separation) of each island into its own buffer j (all
     * zeroed in phase 4); an island has stopped before iteration `it` if some earlier buffer
     * shows min separation >= -3 slop. Buffers of finished iterations are complete after the
     * colour barriers, so no extra barrier per iteration is needed. */
    const float tol = 3.0f * kLinearSlop;
    for (int it = 0; it < sp.pi; ++it) {
        uint32_t* cur = w.isl_minsep + (size_t)it * w.body_cap;
        for (int c = 0; c < ncol; ++c) {
            const int beg = w.col_off[c], end = w.col_off[c + 1];
            for (int k = beg + gtid; k < end; k += gsize) {
                const int isl = w.vc_island[k];
                bool done = false;
                for (int j = 0; j < it && !done; ++j)
                    done = __uint_as_float(w.isl_minsep[(size_t)j * w.body_cap + isl]) <= tol;
                if (done) continue;
                const float ms = solve_position_slot(w, k);
                if (ms < 0.0f) atomicMax(&cur[isl], __float_as_uint(-ms));
            }
            if (!grid_barrier(w)) return;
        }
    }
    /* phase 6a: copy back (synchronize_transform), sleep bookkeeping, clear forces */
    const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
    const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
    for (int b = gtid; b < nb; b += gsize) {
        const uint32_t f = w.b_flags[b];
        if (f & BF_ISLAND) {
            const float4 p = w.b_pos[b];
            const float2 lc = w.b_lc[b];
            Rot q = rot(p.z);
            V2 xp = sub(mk(p.x, p.y), mul(q, mk(lc.x, lc.y)));
            w.b_xf[b] = make_float4(xp.x, xp.y, q.s, q.c);
            if (sp.allow_sleep) {
                float4 v = w.b_vel[b];
                float st;
                if (!(f & BF_AUTO_SLEEP) || v.z * v.z > angTolSqr || v.x * v.x + v.y * v.y > linTolSqr) {
                    st = 0.0f;
                    v.w = 0.0f;
                } else {
                    v.w += h;
                    st = v.w;
                }
                w.b_vel[b] = v;
                atomicMin((unsigned*)&w.isl_sleep[w.b_island[b]], __float_as_uint(st));
            }
        }
        if (sp.auto_clear) w.b_force[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (sp.allow_sleep) {
        if (!grid_barrier(w)) return;
        for (int b = gtid; b < nb; b += gsize) {
            const uint32_t f = w.b_flags[b];
            if (!(f & BF_ISLAND)) continue;
            const int r = w.b_island[b];
            bool solved = false;  /* position_solved: some iteration ended with min separation >= -3 slop */
            for (int j = 0; j < sp.pi && !solved; ++j)
                solved = __uint_as_float(w.isl_minsep[(size_t)j * w.body_cap + r]) <= tol;
            if (solved && w.isl_sleep[r] >= kTimeToSleep) {
                w.b_flags[b] = f & ~BF_AWAKE;
                w.b_vel[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                w.b_force[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
    }
    if (!grid_barrier(w)) return;
    /* phase 6b: synchronize fixtures (private/dynamics/b2_body.rs:455-475) */
    for (int f = gtid; f < w.n_fixtures; f += gsize) {
        const int b = w.f_body[f];
        const uint32_t bf = w.b_flags[b];
        if (!(bf & BF_ISLAND) || is_static(bf)) continue;
        const float4 x = w.b_xf[b];
        Xf xf2;
        xf2.p = mk(x.x, x.y);
        xf2.q.s = x.z;
        xf2.q.c = x.w;
        Xf xf1 = xf2;
        if (bf & BF_AWAKE) {
            const float4 p0 = w.b_pos0[b];
            const float2 lc = w.b_lc[b];
            xf1.q = rot(p0.z);
            xf1.p = sub(mk(p0.x, p0.y), mul(xf1.q, mk(lc.x, lc.y)));
        }
        sync_fixture(w, f, xf1, xf2);
    }
}

__global__ void k_sleep_init(DevWorld w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x)
        w.isl_sleep[b] = kMaxFloat;
}

__global__ void k_set_transform(DevWorld w, int body, float px, float py, float angle) {
    /* B2body::set_transform, private/dynamics/b2_body.rs:418-447 */
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    Xf xf;
    xf.q = rot(angle);
    xf.p = mk(px, py);
    if (gtid == 0) {
        const float2 lc = w.b_lc[body];
        V2 c = mul(xf, mk(lc.x, lc.y));
        w.b_xf[body] = make_float4(px, py, xf.q.s, xf.q.c);
        w.b_pos[body] = make_float4(c.x, c.y, angle, 0.0f);
        w.b_pos0[body] = make_float4(c.x, c.y, angle, 0.0f);
    }
    for (int f = gtid; f < w.n_fixtures; f += gridDim.x * blockDim.x)
        if (w.f_body[f] == body) sync_fixture(w, f, xf, xf);
}

__global__ void k_clear_forces(DevWorld w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x)
        w.b_force[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

/* Blocks of the persistent kernels: one per SM by default (cfg_coop_per_sm = 1). They are bound
 * by grid-barrier latency, which grows with the number of arriving blocks (on the 100k-body scene
 * 152 blocks take 21% less solver time than 304); one block of 256 threads per SM still covers a
 * colour of ~39k slots in a single pass. The autotuner may pick two per SM (both fit at the
 * kernels' register counts). If a block did not fit, the cooperative launch would fail and the
 * step report it. */
int coop_blocks(const void* fn, int num_sms) {
    (void)fn;
    return num_sms;
}

}  // namespace

void launch_islands_and_constraints(const DevWorld& w, const StepParams& sp, cudaStream_t s) {
    const int gb = grid_for(w.n_bodies, kBlock, 152 * 8);
    const int gc = grid_for(w.contact_cap, kBlock, 152 * 8);
    k_island_init<<<gb, kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
    k_island_union<<<gc, kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
    k_island_compress<<<gb, kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
    k_island_mark<<<gb, kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
    uint32_t* flag = w.scan_tmp;                        /* contact_cap */
    uint32_t* pos = w.scan_tmp + w.contact_cap;          /* contact_cap */
    uint32_t* tmp = w.scan_tmp + 2 * (size_t)w.contact_cap;
    k_cons_flags<<<gc, kBlock, 0, s>>>(w, flag); B2G_LAUNCHED(1);
    scan_exclusive_u32(flag, pos, &w.cnt[CNT_CONTACTS], w.contact_cap, tmp, &w.cnt[CNT_CONS], s);
    k_cons_scatter<<<gc, kBlock, 0, s>>>(w, flag, pos); B2G_LAUNCHED(1);
    k_cons_clamp<<<1, 32, 0, s>>>(w); B2G_LAUNCHED(1);
    if (sp.allow_sleep) k_sleep_init<<<gb, kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
}

void launch_colouring(const DevWorld& w, cudaStream_t s, int num_sms) {
    const int blocks = coop_blocks((const void*)k_colour, num_sms) * w.cfg_coop_per_sm;
    DevWorld wc = w;
    void* args[] = {&wc};
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    cudaLaunchCooperativeKernel((const void*)k_colour, dim3(blocks), dim3(kBlock), args, 0, s);
    B2G_LAUNCHED(1);
}

int launch_solver(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms) {
    const int blocks = coop_blocks((const void*)k_solve, num_sms) * w.cfg_coop_per_sm;
    DevWorld wc = w;
    StepParams spc = sp;
    void* args[] = {&wc, &spc};
    B2G_LAUNCHED(1);
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    return (int)cudaLaunchCooperativeKernel((const void*)k_solve, dim3(blocks), dim3(kBlock), args, 0, s);
}

void launch_set_transform(const DevWorld& w, int body, float px, float py, float angle, cudaStream_t s) {
    k_set_transform<<<grid_for(w.n_fixtures, kBlock, 152 * 4), kBlock, 0, s>>>(w, body, px, py, angle); B2G_LAUNCHED(1);
}

void launch_clear_forces(const DevWorld& w, cudaStream_t s) {
    k_clear_forces<<<grid_for(w.n_bodies, kBlock, 152 * 4), kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
}

}  // namespace b2g
