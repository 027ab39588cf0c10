/*
 * k_broadphase.cu — pair finding and contact creation (find_new_contacts).
 *
 * Reference: B2broadPhase::update_pairs (src/b2_broad_phase.rs:200-249) with its query
 * callback (src/private/collision/b2_broad_phase.rs:86-111) over B2dynamicTree, then
 * b2_contact_manager_add_pair (src/private/dynamics/b2_contact_manager.rs:178-302).
 *
 * The reference inserts moved proxies into an incremental AVL-balanced tree and queries
 * it once per moved proxy. Here the tree is a linear BVH, rebuilt when a pass decides so
 * (k_bp_decide: proxies changed on the host, many proxies moved, or the hierarchy is a few
 * passes old) and otherwise kept, with each moved proxy's leaf set to its new fat AABB and its
 * ancestors' boxes grown to cover it (k_bp_update). A rebuild:
 *   1. centre bounds of all fat AABBs (atomic min/max on order-preserving ints),
 *   2. 64-bit keys world << 22 | Morton(11-bit x, 11-bit y), radix-sorted with the
 *      fixture index as payload (worlds occupy disjoint key ranges; a static proxy far
 *      larger than every dynamic one takes key world  world + num_worlds, so grounds and
 *      walls form a small hierarchy of their own instead of inflating every ancestor box;
 *      a single world then sorts 23 key bits, three 8-bit passes; 2048 cells per axis keep a
 *      cell near one body in the densest scenes),
 *   3. Karras (2012) hierarchy over the sorted keys (ties broken by position) — every
 *      internal node stores both children's boxes, and after the refit a four-way record of
 *      its grandchildren, so a traversal step is one 80-byte fetch and four overlap tests,
 *   4. bottom-up refit with per-node arrival counters,
 *   5. one thread per moved proxy walks its world's two subtrees with a short stack and
 *      applies the reference's rule: skip itself; skip a moved partner whose proxy id is
 *      larger (that partner reports the pair); emit (min id, max id).
 * Which pass rebuilds changes only how many nodes a query visits: boxes of internal nodes only
 * have to contain their leaves, and leaves hold the exact fat AABBs.
 * The emitted set equals the reference's: every pair of overlapping fat AABBs with at
 * least one moved proxy, each once (b2_test_overlap is closed, so touching boxes pair).
 * add_pair's rejections run inline (same body, no dynamic body, default filter, edge-edge),
 * and a binary search in the key-sorted contact table drops pairs that already have a
 * live contact. New keys are radix-sorted and merged with the surviving contacts into the
 * second contact buffer, which keeps the table sorted by key = refid_min << kb | refid_max.
 */
#include <climits>

#include "b2g_contact.cuh"

namespace b2g {

namespace {

constexpr int kBlock = 256;
constexpr int kStack = 64;
constexpr int kMortonBits = kKeyMortonBits;  /* 11 bits of cell per axis */
constexpr float kCellMax = 2047.0f;

__device__ __forceinline__ int f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ uint32_t spread16(uint32_t x) {
    x &= 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

/* Rebuild the hierarchy when the host changed proxies (created, destroyed, edited, or the continuous
 * pass moved leaves), when more than a quarter of the proxies moved since the last pass or more than
 * half since the last rebuild (grown boxes make queries visit more nodes), or when the hierarchy is
 * CNT_BP_MAX_AGE passes old (b2g_set_hierarchy_max_age). The decision depends only on the world's own
 * state, so a world and its checkpointed copy decide alike. A repeated pass (the same pass run again
 * after its capacities grew) keeps the decision. */
__global__ void k_bp_decide(DevWorld w, int mode) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int* c = w.cnt;
    const int n = w.n_fixtures;
    /* the pass's counters */
    c[CNT_BOUNDS + 0] = INT_MAX;
    c[CNT_BOUNDS + 1] = INT_MAX;
    c[CNT_BOUNDS + 2] = INT_MIN;
    c[CNT_BOUNDS + 3] = INT_MIN;
    c[CNT_NEW] = 0;
    c[CNT_PAIRS] = 0;
    c[CNT_DYN_EXTENT] = 0;
    c[CNT_BP_VISITS] = 0;
    c[CNT_BP_CANDIDATES] = 0;
    c[CNT_BP_WARP_VISITS] = 0;
    c[CNT_BP_WARP_CHECKS] = 0;
    if (mode == BP_REPEAT) return;
    const int moved = c[CNT_BP_MOVED];
    const long long drift = (long long)c[CNT_BP_DRIFT] + moved;
    const bool rebuild = mode == BP_REBUILD || c[CNT_BP_FORCE] != 0 || c[CNT_BP_NF] != n || c[CNT_BP_AGE] >= c[CNT_BP_MAX_AGE] ||
                         4LL * moved > n || 2LL * drift > n;
    c[CNT_BP_REBUILD] = rebuild ? 1 : 0;
    c[CNT_BP_SORT_N] = rebuild ? n : 0;
    c[CNT_BP_AGE] = rebuild ? 0 : c[CNT_BP_AGE] + 1;
    c[CNT_BP_DRIFT] = rebuild ? 0 : (int)drift;
    c[CNT_BP_NF] = n;
    c[CNT_BP_FORCE] = 0;
    c[CNT_BP_LAST_MOVED] = moved;
    c[CNT_BP_MOVED] = 0;
}

__device__ __forceinline__ bool bp_rebuilding(const DevWorld& w) { return w.cnt[CNT_BP_REBUILD] != 0; }


__global__ void k_bp_bounds(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (!bp_rebuilding(w)) return;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x)
        w.b_rank[b] = INT_MAX;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * w.num_worlds; i += gridDim.x * blockDim.x) {
        w.bp_world_first[i] = -1;
        w.bp_world_root[i] = INT_MIN;
    }
    int mnx = INT_MAX, mny = INT_MAX, mxx = INT_MIN, mxy = INT_MIN, dyn = 0;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < w.n_fixtures; f += gridDim.x * blockDim.x) {
        const float4 a = w.f_fat[f];
        const float cx = 0.5f * (a.x + a.z), cy = 0.5f * (a.y + a.w);
        if (!(cx - cx == 0.0f) || !(cy - cy == 0.0f)) continue;  /* disabled proxies hold infinite boxes */
        if ((w.b_flags[w.f_body[f]] & BF_TYPE_MASK) == BODY_DYNAMIC)
            dyn = max(dyn, __float_as_int(0.5f * fmaxf(a.z - a.x, a.w - a.y)));  /* >= 0: ordered as int */
        const int ix = f2ord(cx), iy = f2ord(cy);
        mnx = min(mnx, ix);
        mny = min(mny, iy);
        mxx = max(mxx, ix);
        mxy = max(mxy, iy);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    for (int o = 16; o > 0; o >>= 1) dyn = max(dyn, __shfl_xor_sync(0xffffffffu, dyn, o));
    /* then over the block's warps, so the five counters take one atomic per block */
    __shared__ int s_red[5][kBlock / 32];
    const int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_red[0][wid] = mnx;
        s_red[1][wid] = mny;
        s_red[2][wid] = mxx;
        s_red[3][wid] = mxy;
        s_red[4][wid] = dyn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
            mnx = min(mnx, s_red[0][i]);
            mny = min(mny, s_red[1][i]);
            mxx = max(mxx, s_red[2][i]);
            mxy = max(mxy, s_red[3][i]);
            dyn = max(dyn, s_red[4][i]);
        }
        atomicMax(&w.cnt[CNT_DYN_EXTENT], dyn);
        atomicMin(&w.cnt[CNT_BOUNDS + 0], mnx);
        atomicMin(&w.cnt[CNT_BOUNDS + 1], mny);
        atomicMax(&w.cnt[CNT_BOUNDS + 2], mxx);
        atomicMax(&w.cnt[CNT_BOUNDS + 3], mxy);
    }
}

__global__ void k_bp_keys(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (!bp_rebuilding(w)) return;
    float lx = 0.0f, ly = 0.0f, sx = 0.0f, sy = 0.0f;
    if (w.cnt[CNT_BOUNDS + 0] != INT_MAX) {
        lx = ord2f(w.cnt[CNT_BOUNDS + 0]);
        ly = ord2f(w.cnt[CNT_BOUNDS + 1]);
        const float ex = ord2f(w.cnt[CNT_BOUNDS + 2]) - lx;
        const float ey = ord2f(w.cnt[CNT_BOUNDS + 3]) - ly;
        sx = ex > 0.0f ? kCellMax / ex : 0.0f;
        sy = ey > 0.0f ? kCellMax / ey : 0.0f;
    }
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < w.n_fixtures; f += gridDim.x * blockDim.x) {
        const float4 a = w.f_fat[f];
        const float cx = 0.5f * (a.x + a.z), cy = 0.5f * (a.y + a.w);
        float qx = (cx - lx) * sx, qy = (cy - ly) * sy;
        qx = (qx - qx == 0.0f) ? fminf(fmaxf(qx, 0.0f), kCellMax) : kCellMax;
        qy = (qy - qy == 0.0f) ? fminf(fmaxf(qy, 0.0f), kCellMax) : kCellMax;
        const uint32_t m = spread16((uint32_t)qx) | (spread16((uint32_t)qy) << 1);
        /* A static proxy much larger than every dynamic one (a ground or a wall) would give all
         * its ancestors a huge box that every query must descend; it goes to its world's second
         * key range (world + num_worlds), a separate small hierarchy that queries also walk. */
        const int b = w.f_body[f];
        uint32_t world = w.b_world[b];
        const float big = 4.0f * __int_as_float(w.cnt[CNT_DYN_EXTENT]);
        if ((w.b_flags[b] & BF_TYPE_MASK) == BODY_STATIC && big > 0.0f &&
            0.5f * fmaxf(a.z - a.x, a.w - a.y) > big)
            world += (uint32_t)w.num_worlds;
        w.bp_key[f] = ((unsigned long long)world << kMortonBits) | m;
        w.bp_val[f] = (uint32_t)f;
    }
}

__device__ __forceinline__ int delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll((long long)(a ^ b));
}

/* Karras, "Maximizing parallelism in the construction of BVHs, octrees, and k-d trees" (HPG 2012) */
__global__ void k_bp_build(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (!bp_rebuilding(w)) return;
    const int n = w.n_fixtures;
    const unsigned long long* k = w.bp_key;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = delta(k, n, i, i - d);
        int lmax = 2;
        while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = delta(k, n, i, j);
        int s = 0;
        int t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int gamma = i + s * d + (d < 0 ? -1 : 0);
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        const int left = (lo == gamma) ? ~gamma : gamma;
        const int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
        w.bp_node_child[i] = make_int2(left, right);
        if (left < 0) w.bp_parent[n - 1 + gamma] = i; else w.bp_parent[gamma] = i;
        if (right < 0) w.bp_parent[n - 1 + gamma + 1] = i; else w.bp_parent[gamma + 1] = i;
        w.bp_flag[i] = 0u;
        /* world root: the node whose leaf range is exactly one world's range */
        const uint32_t wl = (uint32_t)(k[lo] >> kMortonBits), wh = (uint32_t)(k[hi] >> kMortonBits);
        if (wl == wh) {
            const bool first = lo == 0 || (uint32_t)(k[lo - 1] >> kMortonBits) != wl;
            const bool last = hi == n - 1 || (uint32_t)(k[hi + 1] >> kMortonBits) != wl;
            if (first && last) w.bp_world_root[wl] = i;
        }
    }
    /* the leaves: each proxy's box in sorted order, its place, its body's Morton rank */
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t f = w.bp_val[p];
        w.bp_leaf[p] = w.f_fat[f];
        w.f_leaf[f] = p;
        atomicMin(&w.b_rank[w.f_body[f]], p);  /* the body's Morton rank: its first proxy's position */
        const uint32_t wd = (uint32_t)(w.bp_key[p] >> kMortonBits);
        const bool first = p == 0 || (uint32_t)(w.bp_key[p - 1] >> kMortonBits) != wd;
        const bool last = p == n - 1 || (uint32_t)(w.bp_key[p + 1] >> kMortonBits) != wd;
        if (first) w.bp_world_first[wd] = p;
        if (first && last) w.bp_world_root[wd] = ~p;  /* a world with a single proxy */
    }
}


__device__ __forceinline__ float4 box_union(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
}

/* arrival count with release (this thread's box store before it) and acquire (the sibling's after it) */
__device__ __forceinline__ unsigned arrive_acq_rel(unsigned* p) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

/* Bottom-up: each leaf's thread stores its box in its parent's record and arrives; the second of
 * the two children to arrive reads its sibling's box (in L2) and carries the union up. */
__global__ void k_bp_refit(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (!bp_rebuilding(w)) return;
    const int n = w.n_fixtures;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        if (n < 2) break;
        int child = ~p;
        float4 box = w.bp_leaf[p];
        int node = w.bp_parent[n - 1 + p];
        for (int guard = 0; guard < 128; ++guard) {
            const int2 ch = w.bp_node_child[node];
            const bool left = ch.x == child;
            (left ? w.bp_node_b0 : w.bp_node_b1)[node] = box;
            if (arrive_acq_rel(&w.bp_flag[node]) == 0u) break;  /* the sibling finishes this node */
            const float4 sib = __ldcg(&(left ? w.bp_node_b1 : w.bp_node_b0)[node]);
            box = left ? box_union(box, sib) : box_union(sib, box);
            if (node == 0) break;
            child = node;
            node = w.bp_parent[node];
        }
    }
}

__device__ __forceinline__ bool box_overlap(float4 a, float4 b) { return overlap4(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w); }

/* After the refit: each internal node's four-way record, its children's children (a leaf child
 * stands for itself). A traversal then tests four boxes per dependent fetch and descends two
 * levels at a time; the pairs found do not depend on the hierarchy's shape. */
__global__ void k_bp_quad(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (!bp_rebuilding(w)) return;
    const int n = w.n_fixtures;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int2 ch = w.bp_node_child[i];
        const int kids[2] = {ch.x, ch.y};
        const float4 boxes[2] = {w.bp_node_b0[i], w.bp_node_b1[i]};
        int ids[4] = {INT_MIN, INT_MIN, INT_MIN, INT_MIN};
        float4 qb[4];
        int m = 0;
        for (int c = 0; c < 2; ++c) {
            const int k = kids[c];
            if (k < 0) {
                ids[m] = k;
                qb[m++] = boxes[c];
            } else {
                const int2 g = w.bp_node_child[k];
                ids[m] = g.x;
                qb[m++] = w.bp_node_b0[k];
                ids[m] = g.y;
                qb[m++] = w.bp_node_b1[k];
            }
        }
        for (; m < 4; ++m) qb[m] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w.bp_quad_child[i] = make_int4(ids[0], ids[1], ids[2], ids[3]);
        for (int j = 0; j < 4; ++j) w.bp_quad_box[4 * (size_t)i + j] = qb[j];
    }
}

/* componentwise growth of a stored box; returns whether this call changed it */
__device__ __forceinline__ bool grow_lo(float* p, float v) {
    int old = __float_as_int(*(volatile float*)p);
    bool changed = false;
    while (v < __int_as_float(old)) {
        const int prev = atomicCAS((int*)p, old, __float_as_int(v));
        if (prev == old) {
            changed = true;
            break;
        }
        old = prev;
    }
    return changed;
}
__device__ __forceinline__ bool grow_hi(float* p, float v) {
    int old = __float_as_int(*(volatile float*)p);
    bool changed = false;
    while (v > __int_as_float(old)) {
        const int prev = atomicCAS((int*)p, old, __float_as_int(v));
        if (prev == old) {
            changed = true;
            break;
        }
        old = prev;
    }
    return changed;
}
__device__ __forceinline__ bool grow_box(float4* slot, float4 b) {
    const bool x0 = grow_lo(&slot->x, b.x);
    const bool y0 = grow_lo(&slot->y, b.y);
    const bool x1 = grow_hi(&slot->z, b.z);
    const bool y1 = grow_hi(&slot->w, b.w);
    return x0 || y0 || x1 || y1;
}
/* the place of child id in node's four-way record (-1 if absent) */
__device__ __forceinline__ int quad_place(const DevWorld& w, int node, int id) {
    const int4 q = w.bp_quad_child[node];
    return q.x == id ? 0 : q.y == id ? 1 : q.z == id ? 2 : q.w == id ? 3 : -1;
}

/* The contact rows (every pass), then, in a pass that keeps the hierarchy: every moved proxy's leaf
 * takes its new fat AABB exactly (the leaf box, its parent's record of it and the four-way records of
 * its parent and grandparent), and each ancestor's record grows to cover it (the binary record in its
 * parent and the four-way record in its grandparent). A walk stops at the first ancestor whose record already covered the box: whoever grew
 * that record past it carries the growth further up, so when the kernel ends every ancestor covers
 * every leaf below it. */
__global__ void k_bp_update(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    /* every pass: the row index of the key-sorted contact table, c_row[r] = the first contact whose
     * key's high part is proxy id r. Entries of ids with no contact keep stale values; a reader
     * accepts c_row[r] only if that contact's key starts with r, which a stale entry cannot satisfy
     * (ids with contacts are rewritten every pass and the table is sorted). */
    const int nc = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
        const unsigned long long r = w.c.key[i] >> w.key_bits;
        if (i == 0 || (w.c.key[i - 1] >> w.key_bits) != r) w.c_row[r] = i;
        if (i == nc - 1 || (w.c.key[i + 1] >> w.key_bits) != r) w.c_row_end[r] = i + 1;
    }
    if (bp_rebuilding(w)) return;
    const int n = w.n_fixtures;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        if (!w.f_moved[f]) continue;
        const int l = w.f_leaf[f];
        if (l < 0 || l >= n) continue;
        const float4 box = w.f_fat[f];
        w.bp_leaf[l] = box;
        if (n < 2) continue;
        const int n1 = w.bp_parent[n - 1 + l];
        const int2 c1 = w.bp_node_child[n1];
        if (c1.x == ~l) w.bp_node_b0[n1] = box; else w.bp_node_b1[n1] = box;
        int k = quad_place(w, n1, ~l);
        if (k >= 0) w.bp_quad_box[4 * (size_t)n1 + k] = box;
        if (n1 != 0) {
            const int n2 = w.bp_parent[n1];
            k = quad_place(w, n2, ~l);
            if (k >= 0) w.bp_quad_box[4 * (size_t)n2 + k] = box;
        }
        int x = n1;
        for (int guard = 0; guard < 128 && x != 0; ++guard) {
            const int px = w.bp_parent[x];
            const int2 pc = w.bp_node_child[px];
            const bool changed = grow_box(pc.x == x ? &w.bp_node_b0[px] : &w.bp_node_b1[px], box);
            if (px != 0) {
                const int gp = w.bp_parent[px];
                k = quad_place(w, gp, x);
                if (k >= 0) grow_box(&w.bp_quad_box[4 * (size_t)gp + k], box);
            }
            if (!changed) break;
            x = px;
        }
    }
}

__device__ __forceinline__ int lower_bound_u64(const unsigned long long* a, int n, unsigned long long key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* A live contact with this key exists: a search of the key's row of the sorted table instead of the
 * whole table (the check the reference makes by walking body B's contact list,
 * private/dynamics/b2_contact_manager.rs:199-224): a short row is scanned, a long one (a ground
 * touching a whole layer of a pile) is searched by bisection. The row's bounds (c_row, c_row_end)
 * and its first key come from the caller, which loads them for several pairs at a time. */
constexpr int kRowScan = 8;

__device__ __forceinline__ bool contact_exists_from(const DevWorld& w, uint32_t lo, unsigned long long key, int start,
                                                    int end, unsigned long long first, int n_contacts) {
    if (start < 0 || start >= n_contacts || (first >> w.key_bits) != lo) return false;
    if (first >= key) return first == key && !(w.c.flags[start] & CF_DEAD);
    end = min(end, n_contacts);
    int i = start + 1;
    if (end - i <= kRowScan) {
        for (; i < end; ++i) {
            const unsigned long long k = w.c.key[i];
            if (k >= key) return k == key && !(w.c.flags[i] & CF_DEAD);
        }
        return false;
    }
    int hi = end;
    while (i < hi) {
        const int mid = (i + hi) >> 1;
        if (w.c.key[mid] < key) i = mid + 1; else hi = mid;
    }
    return i < end && w.c.key[i] == key && !(w.c.flags[i] & CF_DEAD);
}

/* A slot of a list whose length is *counter, for every lane that executes this together: one atomic
 * per group of lanes (every accepted pair taking a slot with its own atomic on the one counter word
 * serialised them; a pile's traversal accepts tens of thousands per pass) */
__device__ __forceinline__ int agg_slot(int* counter) {
    const unsigned act = __activemask();
    const int lane = (int)(threadIdx.x & 31);
    const int leader = __ffs(act) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(act));
    base = __shfl_sync(act, base, leader);
    return base + __popc(act & ((1u << lane) - 1u));
}

/* add_pair for the pair (f, g) of proxy ids rf, rg with key `key` (lo = the smaller id), whose row
 * in the contact table starts at `start` with key `first` (both read beforehand) */
__device__ void handle_pair(const DevWorld& w, const StepParams& sp, int f, int g, uint32_t rf, uint32_t rg,
                            unsigned long long key, uint32_t lo, int start, int end, unsigned long long first,
                            int n_contacts) {
    if (sp.record_pairs) {
        const int slot = agg_slot(&w.cnt[CNT_PAIRS]);
        if (slot < w.pair_cap) w.pairs[slot] = make_uint2((uint32_t)min(f, g), (uint32_t)max(f, g));
        else atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_RECORD_OVERFLOW);
    }
    /* most overlapping pairs already have a contact: test that first (the order of the tests
     * does not change which pairs are added) */
    if (contact_exists_from(w, lo, key, start, end, first, n_contacts)) return;
    /* add_pair: fixture A is the one with the smaller proxy id */
    int fa, fb;
    if (!pair_accept(w, rf < rg ? f : g, rf < rg ? g : f, fa, fb, !sp.custom_filter)) return;
    const int slot = agg_slot(&w.cnt[CNT_NEW]);
    if (slot < w.pair_cap) {
        w.n_key[slot] = key;
        w.n_fix[slot] = make_int2(fa, fb);
        w.n_idx[slot] = (uint32_t)slot;
    } else {
        atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_PAIR_OVERFLOW);
    }
}

/* The partner checks of up to kCheckBatch queued leaves of one lane (entries i0, i0 + 32, ...): the
 * reference's rules (skip itself; skip a moved partner with the larger proxy id, which reports the
 * pair) and add_pair. Each check is a chain of dependent loads (partner, its proxy id and moved
 * flag, the contact row's bounds, its first key), so the batch issues each link of all its chains together.
 * Returns the entries checked. */
constexpr int kCheckBatch = 4;

__device__ __forceinline__ unsigned check_batch(const DevWorld& w, const StepParams& sp, const uint2* queue, int i0, int nq,
                                                int n_contacts) {
    int ff[kCheckBatch], g[kCheckBatch];
    bool ok[kCheckBatch];
    unsigned n = 0;
#pragma unroll
    for (int k = 0; k < kCheckBatch; ++k) {
        const int i = i0 + 32 * k;
        ok[k] = i < nq;
        const uint2 e = ok[k] ? queue[i] : make_uint2(0u, 0u);
        ff[k] = (int)e.x;
        g[k] = ok[k] ? (int)w.bp_val[e.y] : 0;
        n += ok[k] ? 1u : 0u;
    }
    uint32_t rf[kCheckBatch], rg[kCheckBatch];
#pragma unroll
    for (int k = 0; k < kCheckBatch; ++k) {
        rf[k] = ok[k] ? w.f_refid[ff[k]] : 0u;
        rg[k] = ok[k] ? w.f_refid[g[k]] : 0u;
        const bool moved = ok[k] && w.f_moved[g[k]] != 0;
        ok[k] = ok[k] && g[k] != ff[k] && !(moved && rg[k] > rf[k]);
    }
    uint32_t lo[kCheckBatch];
    int start[kCheckBatch], end[kCheckBatch];
#pragma unroll
    for (int k = 0; k < kCheckBatch; ++k) {
        lo[k] = rf[k] < rg[k] ? rf[k] : rg[k];
        start[k] = ok[k] ? w.c_row[lo[k]] : -1;
        end[k] = ok[k] ? w.c_row_end[lo[k]] : -1;
    }
    unsigned long long first[kCheckBatch];
#pragma unroll
    for (int k = 0; k < kCheckBatch; ++k)
        first[k] = ok[k] && start[k] >= 0 && start[k] < n_contacts ? w.c.key[start[k]] : ~0ull;
#pragma unroll
    for (int k = 0; k < kCheckBatch; ++k) {
        if (!ok[k]) continue;
        const uint32_t hi = rf[k] < rg[k] ? rg[k] : rf[k];
        const unsigned long long key = ((unsigned long long)lo[k] << w.key_bits) | hi;
        handle_pair(w, sp, ff[k], g[k], rf[k], rg[k], key, lo[k], start[k], end[k], first[k], n_contacts);
    }
    return n;
}

/* One lane per moved proxy starts a walk of the hierarchies, and a warp walks in step:
 *  - a lane only queues the leaves its query box overlaps (in shared memory), and whenever a warp
 *    has 32 or more queued the whole warp checks them, one leaf per lane (the partner rules, the
 *    existing-contact row scan and add_pair's filters are chains of dependent loads);
 *  - a lane whose walk is done takes over the oldest pending node of a lane with two or more,
 *    with that lane's query box, so a warp's rounds follow its total work rather than its longest
 *    walk. */
constexpr int kLeafQueue = 224;  /* 31 left over + 32 lanes x 4 leaves in one round, or the setup's
                                    2 single-proxy roots per lane */

__global__ void __launch_bounds__(kBlock) k_bp_traverse(DevWorld w, StepParams sp) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    __shared__ uint2 s_queue[kBlock / 32][kLeafQueue];
    __shared__ int s_give_node[kBlock / 32][32];
    __shared__ int s_give_f[kBlock / 32][32];
    __shared__ float4 s_give_q[kBlock / 32][32];
    const int n = w.n_fixtures;
    const int n_contacts = w.cnt[CNT_CONTACTS];
    const uint32_t nw = (uint32_t)w.num_worlds;
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
    uint2* queue = s_queue[wq];
    const int stride = gridDim.x * blockDim.x;
    unsigned visits = 0, candidates = 0;  /* this lane's node fetches and leaf checks (traffic counters) */
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int p = base + lane;
        int f = -1;
        if (p < n) {
            f = (int)w.bp_val[p];
            if (!w.f_moved[f]) f = -1;
        }
        int stack[kStack];
        int bot = 0, top = 0;  /* pending nodes [bot, top) of the current query */
        int found[6];
        int nfound = 0;
        float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (f >= 0) {
            q = w.bp_leaf[p];
            uint32_t wd = (uint32_t)(w.bp_key[p] >> kMortonBits);
            if (wd >= nw) wd -= nw;
            /* the world's hierarchy and the one of its large static proxies */
            for (int h = 0; h < 2; ++h) {
                const int root = w.bp_world_root[wd + (h ? nw : 0u)];
                if (root == INT_MIN) continue;
                if (root < 0) {  /* a single proxy */
                    if (box_overlap(w.bp_leaf[~root], q)) found[nfound++] = ~root;
                } else {
                    stack[top++] = root;
                }
            }
        }
        int nq = 0;
        /* queue the leaves found so far: a warp prefix sum gives each lane its place */
        auto enqueue = [&]() {
            const unsigned finders = __ballot_sync(full, nfound > 0);
            if (finders == 0u) return;  /* most steps of a walk find no leaf */
            int incl = nfound;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(full, incl, o);
                if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(full, incl, 31);
            for (int i = 0; i < nfound; ++i) queue[nq + incl - nfound + i] = make_uint2((uint32_t)f, (uint32_t)found[i]);
            nfound = 0;
            nq += total;
        };
        enqueue();  /* single-proxy roots, before this lane may take over another query */
        for (;;) {
            /* idle lanes take the oldest pending node of lanes with two or more */
            const unsigned idle = __ballot_sync(full, top == bot);
            const unsigned donors = __ballot_sync(full, top - bot >= 2);
            if (idle != 0u && donors != 0u) {
                const int pairs = min(__popc(idle), __popc(donors));
                if ((donors >> lane) & 1u) {
                    const int r = __popc(donors & lt);
                    if (r < pairs) {
                        s_give_node[wq][r] = stack[bot++];
                        s_give_f[wq][r] = f;
                        s_give_q[wq][r] = q;
                    }
                }
                __syncwarp();
                if ((idle >> lane) & 1u) {
                    const int r = __popc(idle & lt);
                    if (r < pairs) {
                        f = s_give_f[wq][r];
                        q = s_give_q[wq][r];
                        bot = 0;
                        top = 0;
                        stack[top++] = s_give_node[wq][r];
                    }
                }
                __syncwarp();
            }
            if (top > bot) {
                ++visits;
                const int node = stack[--top];
                const int4 ch = w.bp_quad_child[node];
                const float4* qb = w.bp_quad_box + 4 * (size_t)node;
                const float4 bx[4] = {qb[0], qb[1], qb[2], qb[3]};
                const int kids[4] = {ch.x, ch.y, ch.z, ch.w};
                for (int c = 0; c < 4; ++c) {
                    if (kids[c] == INT_MIN || !box_overlap(bx[c], q)) continue;
                    const int id = kids[c];
                    if (id < 0) {
                        found[nfound++] = ~id;
                    } else if (top < kStack) {
                        stack[top++] = id;
                    } else {
                        atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_STACK_OVERFLOW);
                    }
                }
                if (top == bot) bot = top = 0;
            }
            enqueue();
            const bool more = __any_sync(full, top > bot);
            if (nq >= 32 || (!more && nq > 0)) {
                __syncwarp();
                for (int i0 = lane; i0 < nq; i0 += 32 * kCheckBatch)
                    candidates += check_batch(w, sp, queue, i0, nq, n_contacts);
                __syncwarp();
                nq = 0;
            }
            if (!more) break;
        }
    }
    visits = __reduce_add_sync(0xffffffffu, visits);
    candidates = __reduce_add_sync(0xffffffffu, candidates);
    if (lane == 0 && (visits | candidates)) {
        atomicAdd((unsigned*)&w.cnt[CNT_BP_VISITS], visits);
        atomicAdd((unsigned*)&w.cnt[CNT_BP_CANDIDATES], candidates);
        atomicMax((unsigned*)&w.cnt[CNT_BP_WARP_VISITS], visits);
        atomicMax((unsigned*)&w.cnt[CNT_BP_WARP_CHECKS], candidates);
    }
}

/* the moved flags are consumed; the colouring's rank weights start from zero (they are indexed by
 * Morton rank, of which there are as many as proxies) */
__global__ void k_bp_clear_moved(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < w.n_fixtures; f += gridDim.x * blockDim.x) {
        w.f_moved[f] = 0;
        w.rank_x[f] = 0ull;
    }
}


/* ---- merge of surviving contacts and new contacts (both key-sorted) ---- */
__global__ void k_merge_flags(DevWorld w, uint32_t* flag) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flag[i] = (w.c.flags[i] & CF_DEAD) ? 0u : 1u;
}

__global__ void k_merge_old(DevWorld w, const uint32_t* flag, const uint32_t* rank) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    const int n = w.cnt[CNT_CONTACTS];
    const int nn = min(w.cnt[CNT_NEW], w.pair_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        const int pos = (int)rank[i] + lower_bound_u64(w.n_key, nn, w.c.key[i]);
        if (pos < w.contact_cap) copy_contact(w.c, i, w.c_alt, pos);
        else atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_CONTACT_OVERFLOW);
    }
}

/* b2_contact_create + B2contact::new (private/dynamics/b2_contact.rs:11-60): mixing laws of src/b2_contact.rs:29-46 */
__global__ void k_merge_new(DevWorld w, const uint32_t* rank) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    const int n = w.cnt[CNT_CONTACTS];
    const int nn = min(w.cnt[CNT_NEW], w.pair_cap);
    const int alive = w.cnt[CNT_ALIVE];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nn; j += gridDim.x * blockDim.x) {
        const unsigned long long key = w.n_key[j];
        const int2 fx = w.n_fix[w.n_idx[j]];
        const int at = lower_bound_u64(w.c.key, n, key);
        const int before = at < n ? (int)rank[at] : alive;
        const int pos = j + before;
        if (pos >= w.contact_cap) {
            atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_CONTACT_OVERFLOW);
            continue;
        }
        init_contact(w, w.c_alt, pos, key, fx);
    }
}

__global__ void k_merge_finish(DevWorld w) {
    pdl_entry();
    B2G_RETURN_IF_ABORTED(w);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.cnt[CNT_MERGE_FROM] = w.cnt[CNT_CONTACTS];
        int total = w.cnt[CNT_ALIVE] + min(w.cnt[CNT_NEW], w.pair_cap);
        if (total > w.contact_cap) {
            total = w.contact_cap;
            atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_CONTACT_OVERFLOW);
        }
        w.cnt[CNT_CONTACTS] = total;
    }
}

__global__ void k_touch_all(DevWorld w) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < w.n_fixtures; f += gridDim.x * blockDim.x)
        w.f_moved[f] = w.f_refid[f] != 0xffffffffu ? 1 : 0;
}

}  // namespace

void launch_touch_all_proxies(const DevWorld& w, cudaStream_t s) {
    k_touch_all<<<grid_for(w.n_fixtures, kBlock, w.num_sms * 8), kBlock, 0, s>>>(w);
    B2G_LAUNCHED(1);
}

/* Runs update_pairs + add_pair and merges: the caller swaps w.c and w.c_alt afterwards. */
void launch_broadphase(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms,
                       const std::function<void(int)>& mark, int mode) {
    const int n = w.n_fixtures;
    const int gf = grid_for(n, kBlock, num_sms * 8);
    launch_pdl(k_bp_decide, 1, 32, 0, s, w, mode); B2G_LAUNCHED(1);
    if (n > 0) {
        launch_pdl(k_bp_bounds, gf, kBlock, 0, s, w); B2G_LAUNCHED(1);
        launch_pdl(k_bp_keys, gf, kBlock, 0, s, w); B2G_LAUNCHED(1);
        radix_sort_pairs_coop(w.bp_key, w.bp_val, w.bp_key_alt, w.bp_val_alt, &w.cnt[CNT_BP_SORT_N], n,
                              kMortonBits + w.morton_world_bits, w.sort_hist, w.cnt, s, num_sms, true);
        if (mark) mark(0);
        launch_pdl(k_bp_build, gf, kBlock, 0, s, w); B2G_LAUNCHED(1);
        launch_pdl(k_bp_refit, gf, kBlock, 0, s, w); B2G_LAUNCHED(1);
        if (n > 1) {
            launch_pdl(k_bp_quad, grid_for(n - 1, kBlock, num_sms * 8), kBlock, 0, s, w); B2G_LAUNCHED(1);
        }
        launch_pdl(k_bp_update, grid_for(std::max(n, w.contact_cap), kBlock, num_sms * 8), kBlock, 0, s, w);
        B2G_LAUNCHED(1);
        if (mark) mark(1);
        const int tb = w.cfg_traverse_block;
        launch_pdl(k_bp_traverse, grid_for(n, tb, num_sms * 2048 / tb), tb, 0, s, w, sp); B2G_LAUNCHED(1);
        launch_pdl(k_bp_clear_moved, gf, kBlock, 0, s, w); B2G_LAUNCHED(1);
    }
    if (mark) mark(2);
    /* sort new keys; payload = emission slot */
    radix_sort_pairs_coop(w.n_key, w.n_idx, w.n_key_alt, w.n_idx_alt, &w.cnt[CNT_NEW], w.pair_cap, 2 * w.key_bits,
                          w.sort_hist, w.cnt, s, num_sms);
    uint32_t* flag = w.scan_tmp;
    uint32_t* rank = w.scan_tmp + w.contact_cap;
    uint32_t* tmp = w.scan_tmp + 2 * (size_t)w.contact_cap;
    const int gc = grid_for(w.contact_cap, kBlock, num_sms * 8);
    launch_pdl(k_merge_flags, gc, kBlock, 0, s, w, flag); B2G_LAUNCHED(1);
    scan_exclusive_u32(flag, rank, &w.cnt[CNT_CONTACTS], w.contact_cap, tmp, &w.cnt[CNT_ALIVE], s);
    launch_pdl(k_merge_old, gc, kBlock, 0, s, w, (const uint32_t*)flag, (const uint32_t*)rank); B2G_LAUNCHED(1);
    launch_pdl(k_merge_new, grid_for(w.pair_cap, kBlock, num_sms * 8), kBlock, 0, s, w, (const uint32_t*)rank);
    B2G_LAUNCHED(1);
    launch_pdl(k_merge_finish, 1, 32, 0, s, w); B2G_LAUNCHED(1);
}

}  // namespace b2g
