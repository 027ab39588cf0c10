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
#include "b2g_joint.cuh"
#include "b2g_solver_math.cuh"
#include "b2g_sync.cuh"

namespace b2g {

namespace {

constexpr int kBlock = 256;
static_assert(kBlock == kMaxColours, "the colouring scans one histogram row of kMaxColours per block");

__device__ __forceinline__ bool is_dynamic(uint32_t flags) { return (flags & BF_TYPE_MASK) == BODY_DYNAMIC; }
__device__ __forceinline__ bool is_static(uint32_t flags) { return (flags & BF_TYPE_MASK) == BODY_STATIC; }

/* Atomics on per-island words, aggregated over the lanes of a warp that execute them together: a
 * pile that is one large island would otherwise send every constraint's update to the same word,
 * and same-address atomics are serialised. Each lane calls once; the lanes with the same island
 * combine their values and one of them updates the word (a zero value updates nothing). */
__device__ __forceinline__ void agg_atomic_max(unsigned* words, int key, unsigned v) {
    const unsigned peers = __match_any_sync(__activemask(), key);
    const unsigned m = __reduce_max_sync(peers, v);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && m != 0u) atomicMax(&words[key], m);
}
__device__ __forceinline__ void agg_atomic_or(unsigned* words, int key, unsigned v) {
    const unsigned peers = __match_any_sync(__activemask(), key);
    const unsigned m = __reduce_or_sync(peers, v);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && m != 0u) atomicOr(&words[key], m);
}
__device__ __forceinline__ void agg_atomic_min(unsigned* words, int key, unsigned v) {
    const unsigned peers = __match_any_sync(__activemask(), key);
    const unsigned m = __reduce_min_sync(peers, v);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicMin(&words[key], m);
}
/* a counter incremented by every lane that executes this */
__device__ __forceinline__ void agg_increment(int* counter) {
    const unsigned act = __activemask();
    if ((int)(threadIdx.x & 31) == __ffs(act) - 1) atomicAdd(counter, __popc(act));
}

/* ---------------- islands ---------------- */
/* Other SMs relink roots during the union pass, and a link cached in this SM's L1 may still show
 * a root that is no longer one: a find can stop early, at an ancestor. uf_union therefore goes on
 * from the parent a failed link returns (read in L2), so every retry climbs at least one link. */
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

/* link the larger root under the smaller; a failed link continues from the parent it found */
__device__ __forceinline__ void uf_union(int* parent, int a, int b) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    for (int guard = 0; guard < 1 << 20 && a != b; ++guard) {
        const int hi = a > b ? a : b, lo = a > b ? b : a;
        const int old = atomicCAS(&parent[hi], hi, lo);
        if (old == hi) return;
        a = uf_find(parent, old);
        b = uf_find(parent, lo);
    }
}

__device__ __forceinline__ bool contact_is_constraint(uint32_t cf) {
    return (cf & (CF_TOUCHING | CF_ENABLED | CF_DEAD | CF_SENSOR)) == (CF_TOUCHING | CF_ENABLED);
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

/* Block-wide exclusive scan of one int per thread (blockDim.x == kBlock); *total gets the sum. */
__device__ __forceinline__ int block_scan_excl(int v, int* total) {
    __shared__ int s_warp[kBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    int base = 0, tot = 0;
    for (int i = 0; i < kBlock / 32; ++i) {
        const int t = s_warp[i];
        if (i < wid) base += t;
        tot += t;
    }
    __syncthreads();
    *total = tot;
    return base + x - v;
}

/* Block-wide exclusive scan of one 64-bit value per thread; *total gets the sum. */
__device__ __forceinline__ unsigned long long block_scan_excl64(unsigned long long v, unsigned long long* total) {
    __shared__ unsigned long long s_warp64[kBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp64[wid] = x;
    __syncthreads();
    unsigned long long base = 0, tot = 0;
    for (int i = 0; i < kBlock / 32; ++i) {
        const unsigned long long t = s_warp64[i];
        if (i < wid) base += t;
        tot += t;
    }
    __syncthreads();
    *total = tot;
    return base + x - v;
}

constexpr uint32_t kStampMask = 0x1ffffffu;  /* colouring stamps kept in contacts: 25 bits */

/* The last colouring rounds in one block (block 0), on the listed uncoloured constraints: the
 * rounds of k_colour with block barriers. Offers of both round parities at the listed
 * constraints' bodies are cleared first (earlier rounds may have left them). Returns the next
 * round number and records the rounds. */
__device__ int colour_tail(const DevWorld& w, int round) {
    __shared__ int s_list[kColourTail];
    __shared__ int s_left[2];
    const int m = min(w.cnt[CNT_TAIL], kColourTail);
    const size_t bc = (size_t)w.body_cap;
    const unsigned long long kNone = ~0ull;
    for (int i = threadIdx.x; i < m; i += blockDim.x) s_list[i] = w.col_tail[i];
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int k = s_list[i];
        const int2 bd = w.c.body[w.cons_contact[k]];
        const size_t cm = w.cons_part[k] < 0 ? bc : 0;
        for (int par = 0; par < 2; ++par) {
            w.b_cmin[(size_t)par * 2 * bc + cm + bd.x] = kNone;
            w.b_cmin[(size_t)par * 2 * bc + cm + bd.y] = kNone;
        }
    }
    if (threadIdx.x == 0) s_left[0] = s_left[1] = 0;
    __syncthreads();
    int r = round;
    for (;;) {
        if (r >= kMaxColours - kFirstFitColours) {
            for (int i = threadIdx.x; i < m; i += blockDim.x)
                if (w.cons_colour[s_list[i]] < 0) w.cons_colour[s_list[i]] = kMaxColours - 1;
            if (threadIdx.x == 0) atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_COLOUR_OVERFLOW);
            break;
        }
        unsigned long long* offer = w.b_cmin + (size_t)(r & 1) * 2 * bc;
        unsigned long long* stale = w.b_cmin + (size_t)((r + 1) & 1) * 2 * bc;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const int k = s_list[i];
            const int2 bd = w.c.body[w.cons_contact[k]];
            const size_t cm = w.cons_part[k] < 0 ? bc : 0;
            if (r > round) {
                stale[cm + bd.x] = kNone;
                stale[cm + bd.y] = kNone;
            }
            if (w.cons_colour[k] >= 0) continue;
            const unsigned long long key = ((unsigned long long)hash32((uint32_t)k) << 32) | (uint32_t)k;
            if (is_dynamic(w.b_flags[bd.x])) atomicMin(&offer[cm + bd.x], key);
            if (is_dynamic(w.b_flags[bd.y])) atomicMin(&offer[cm + bd.y], key);
        }
        if (threadIdx.x == 0) s_left[(r + 1) & 1] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const int k = s_list[i];
            if (w.cons_colour[k] >= 0) continue;
            const int2 bd = w.c.body[w.cons_contact[k]];
            const size_t cm = w.cons_part[k] < 0 ? bc : 0;
            const unsigned long long key = ((unsigned long long)hash32((uint32_t)k) << 32) | (uint32_t)k;
            const bool da = is_dynamic(w.b_flags[bd.x]), db = is_dynamic(w.b_flags[bd.y]);
            const bool winA = !da || offer[cm + bd.x] == key;
            const bool winB = !db || offer[cm + bd.y] == key;
            if (winA && winB) {
                const unsigned long long used =
                    (da ? w.b_cmask[cm + bd.x] : 0ull) | (db ? w.b_cmask[cm + bd.y] : 0ull);
                int colour;
                if (~used != 0ull) {
                    colour = __ffsll((long long)~used) - 1;
                    const unsigned long long bit = 1ull << colour;
                    if (da) w.b_cmask[cm + bd.x] |= bit;
                    if (db) w.b_cmask[cm + bd.y] |= bit;
                } else {
                    colour = kFirstFitColours + r;
                    if (colour >= kMaxColours) {
                        colour = kMaxColours - 1;
                        atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_COLOUR_OVERFLOW);
                    }
                }
                w.cons_colour[k] = colour;
            } else {
                atomicAdd(&s_left[r & 1], 1);
            }
        }
        __syncthreads();
        const int left = s_left[r & 1];
        __syncthreads();  /* every thread has read it before the next round clears the other counter */
        ++r;
        if (left == 0) break;
    }
    if (threadIdx.x == 0) w.cnt[CNT_ROUNDS] = r;
    return r;
}

/* Colouring. Constraints are of two classes. With the part-local solve, the dynamic bodies are
 * split into parts (one per solver block, by Morton rank); a constraint whose dynamic bodies all
 * lie in one part is interior, the others are boundary. Interior constraints are solved by their
 * part's block alone and boundary ones in grid-wide colour sweeps afterwards, so only constraints
 * of the same class must differ in colour where they share a dynamic body: each class has its
 * own colour masks and priority offers, and the sparse boundary class needs few colours. Without
 * parts every constraint is boundary (one grid-wide colouring).
 * A constraint of the previous colouring that keeps its class keeps its first-fit colour (stored
 * in its contact with that colouring's stamp and class): the previous colours of a class were a
 * proper colouring of its constraints, so any subset of them still is. Only the others are
 * coloured, by Jones-Plassmann rounds (hash priorities; a local minimum at both of its dynamic
 * bodies takes the lowest colour free at both), so a step whose contacts persist needs one or
 * two rounds instead of one per colour.
 * Slots are then ordered part by part, each part by colour, then the boundary colours: solving
 * the parts concurrently is solving them one after the other, as no two parts share a dynamic
 * body, so this slot order is the sequential solve order. */
__global__ void __launch_bounds__(kBlock) k_colour(DevWorld w, int nparts) {
    B2G_RETURN_IF_ABORTED(w);
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    const int n = w.cnt[CNT_CONS];
    const int nf = w.n_fixtures;
    const int P = (nf > 0 && nparts <= kMaxParts && nparts <= (int)gridDim.x) ? nparts : 0;
    const size_t bc = (size_t)w.body_cap;
    const unsigned long long kNone = ~0ull;
    const uint32_t stamp = (uint32_t)w.cnt[CNT_COLOURINGS] & kStampMask;  /* the previous colouring's */
    /* offers are double-buffered by round parity: round r offers into buffer r & 1, and the
     * entries of buffer (r - 1) & 1 are reset during round r, so a round needs two barriers */
    for (int b = gtid; b < w.n_bodies; b += gsize) {
        for (int j = 0; j < 4; ++j) w.b_cmin[j * bc + b] = kNone;
        w.b_cmask[b] = 0ull;
        w.b_cmask[bc + b] = 0ull;
    }
    /* every 16th colouring starts afresh, so kept colours do not stay fragmented after the
     * contact graph has changed (a fresh colouring of a settled stack needs fewer colours) */
    const bool keep = stamp != 0u && (stamp & 15u) != 0u;
    /* the partition is made afresh every 4th colouring (and when the part or proxy count changed)
     * and kept in between: a body stays in its part, and a body outside the partition goes to the
     * part whose rank range its Morton rank falls in. (Kept colours stay proper across a new
     * partition: interior constraints that share a body are always in the same part.) */
    const bool rebalance = P > 0 && ((stamp & 3u) == 0u || w.cnt[CNT_PART_P] != P || w.cnt[CNT_PART_NF] != nf);
    int ncache = w.cnt[CNT_PART_NCACHE];  /* read before any barrier; a rebalance rewrites it below */
    if (rebalance) {
        /* Parts of equal work: weigh each Morton rank by the constraint endpoints of its body and
         * cut the weight prefix into P equal ranges. rank_x was zeroed by the broadphase. */
        for (int k = gtid; k < n; k += gsize) {
            const int2 bd = w.c.body[w.cons_contact[k]];
            if (is_dynamic(w.b_flags[bd.x]) && w.b_rank[bd.x] < nf) atomicAdd(&w.rank_x[w.b_rank[bd.x]], 1ull << 32);
            if (is_dynamic(w.b_flags[bd.y]) && w.b_rank[bd.y] < nf) atomicAdd(&w.rank_x[w.b_rank[bd.y]], 1ull << 32);
        }
        for (int q = gtid; q < P; q += gsize) {
            w.part_cbeg[q] = 0;
            w.part_cend[q] = 0;
            w.part_rbeg[q] = INT_MAX;
        }
        if (!grid_barrier(w)) return;
        /* each block scans its chunk of ranks: (weight << 32 | has weight), exclusive */
        const int chunk = (nf + (int)gridDim.x - 1) / (int)gridDim.x;
        const int r0 = min(nf, (int)blockIdx.x * chunk), r1 = min(nf, r0 + chunk);
        unsigned long long carry = 0;
        for (int base = r0; base < r1; base += blockDim.x) {
            const int r = base + threadIdx.x;
            unsigned long long v = r < r1 ? w.rank_x[r] : 0ull;
            v += v ? 1ull : 0ull;
            unsigned long long tot;
            const unsigned long long ex = block_scan_excl64(v, &tot);
            if (r < r1) w.rank_x[r] = carry + ex;
            carry += tot;
        }
        if (threadIdx.x == 0) w.blk_tot[blockIdx.x] = carry;
        if (!grid_barrier(w)) return;
        unsigned long long before = 0, all = 0;
        {
            unsigned long long mine = 0, every = 0;
            for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
                const unsigned long long t = w.blk_tot[q];
                if (q < (int)blockIdx.x) mine += t;
                every += t;
            }
            block_scan_excl64(mine, &before);
            block_scan_excl64(every, &all);
        }
        const unsigned long long wtot = all >> 32;
        /* A batch of worlds cuts only at world boundaries: a world's bodies all take the part of the
         * weight prefix at the world's first rank (ranks are grouped by world), so no constraint
         * joins two parts, there are no boundary colours, and the parts never wait for each other.
         * That needs the prefix at any rank: the chunks' prefixes are made global first. */
        const bool aligned = w.num_worlds > 1;
        if (aligned) {
            for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) w.rank_x[r] += before;
            if (!grid_barrier(w)) return;
        }
        const unsigned long long base_x = aligned ? 0ull : before;
        for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
            const unsigned long long x = base_x + w.rank_x[r];
            const unsigned long long x1 = r + 1 < r1 ? base_x + w.rank_x[r + 1] : before + carry;
            if ((uint32_t)x1 == (uint32_t)x || wtot == 0ull) continue;  /* no constraint at this rank */
            unsigned long long px = x;
            if (aligned) {
                const int first = w.bp_world_first[(uint32_t)(w.bp_key[r] >> kKeyMortonBits)];
                if (first >= 0 && first <= r) px = w.rank_x[first];
            }
            const int part = min(P - 1, (int)(((px >> 32) * (unsigned long long)P) / wtot));
            const int c = (int)(uint32_t)x;
            if (c >= nf) continue;  /* cannot happen: at most one constraint body per rank */
            const int b = w.f_body[w.bp_val[r]];
            w.b_part[b] = part;
            w.b_cidx[b] = c;
            w.cache_body[c] = b;
        }
        if (!grid_barrier(w)) return;
        /* each part's range of constraint bodies */
        ncache = min(nf, (int)(uint32_t)all);
        for (int c = gtid; c < ncache; c += gsize) {
            const int part = w.b_part[w.cache_body[c]];
            if (c == 0 || w.b_part[w.cache_body[c - 1]] != part) {
                w.part_cbeg[part] = c;
                int rb = w.b_rank[w.cache_body[c]];
                if (w.num_worlds > 1) {  /* whole worlds: the range starts at the world's first rank */
                    const int first = w.bp_world_first[(uint32_t)(w.bp_key[rb] >> kKeyMortonBits)];
                    if (first >= 0 && first <= rb) rb = first;
                }
                if (part > 0) w.part_rbeg[part] = rb;
            }
            if (c == ncache - 1 || w.b_part[w.cache_body[c + 1]] != part) w.part_cend[part] = c + 1;
        }
        if (gtid == 0) {
            w.cnt[CNT_PART_NCACHE] = ncache;
            w.cnt[CNT_PART_NF] = nf;
            w.cnt[CNT_PART_P] = P;
        }
    }
    if (gtid == 0 && P == 0) w.cnt[CNT_PART_P] = 0;
    /* a body's part: its own if the partition holds it, else the part whose rank range its
     * current Morton rank falls in (the block of that part then reads it in global memory) */
    auto part_of = [&](int b) {
        const int c = w.b_cidx[b];
        if (c >= 0 && c < ncache && w.cache_body[c] == b) return w.b_part[b];
        const int r = w.b_rank[b];
        if (r >= nf) return -2;
        int lo = 0, hi = P - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (w.part_rbeg[mid] <= r) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    };
    for (int k = gtid; k < n; k += gsize) {
        const int ci = w.cons_contact[k];
        int part = -1;
        if (P > 0) {
            const int2 bd = w.c.body[ci];
            const bool da = is_dynamic(w.b_flags[bd.x]), db = is_dynamic(w.b_flags[bd.y]);
            if (P == 1) {
                part = 0;  /* one part holds everything; bodies outside its cache stay in global memory */
            } else {
                const int pa = !da ? -1 : part_of(bd.x);
                const int pb = !db ? -1 : part_of(bd.y);
                part = !da ? pb : (!db ? pa : (pa == pb ? pa : -1));
                if (part < 0) part = -1;
            }
        }
        w.cons_part[k] = part;
        const uint32_t cls = part < 0 ? 1u : 0u;
        const uint32_t kept = w.c.mids[ci].w;
        w.cons_colour[k] = (keep && (kept >> 7) == stamp && ((kept >> 6) & 1u) == cls) ? (int)(kept & 63u) : -1;
    }
    for (int c = gtid; c < (P + 1) * kMaxColours; c += gsize) w.col_hist[c] = 0;
    if (!grid_barrier(w)) return;
    /* the kept colours are taken at their bodies */
    for (int k = gtid; k < n; k += gsize) {
        const int c = w.cons_colour[k];
        if (c < 0) continue;
        const int2 bd = w.c.body[w.cons_contact[k]];
        const size_t cm = w.cons_part[k] < 0 ? bc : 0;
        const unsigned long long bit = 1ull << c;
        if (is_dynamic(w.b_flags[bd.x])) atomicOr(&w.b_cmask[cm + bd.x], bit);
        if (is_dynamic(w.b_flags[bd.y])) atomicOr(&w.b_cmask[cm + bd.y], bit);
    }
    if (gtid == 0) {
        /* two "still uncoloured" counters alternate by round parity: round r counts into
         * [r & 1] and reads the previous round's result from [(r + 1) & 1] */
        w.cnt[CNT_UNCOLOURED] = 0;
        w.cnt[CNT_UNCOLOURED + 1] = n;
        w.cnt[CNT_ROUNDS] = 0;
        w.cnt[CNT_TAIL] = 0;
    }
    if (!grid_barrier(w)) return;
    int round = 0;
    for (;;) {
        const int remaining = ((volatile int*)w.cnt)[CNT_UNCOLOURED + ((round + 1) & 1)];
        if (remaining <= 0) break;
        if (remaining <= kColourTail) {
            /* Few left: list them and let one block finish the rounds with block barriers. Its
             * rounds are the same rounds (priorities, first fit, overflow colours by round). */
            for (int k = gtid; k < n; k += gsize)
                if (w.cons_colour[k] < 0) {
                    const int at = atomicAdd(&w.cnt[CNT_TAIL], 1);
                    if (at < kColourTail) w.col_tail[at] = k;
                }
            if (!grid_barrier(w)) return;
            if (blockIdx.x == 0) round = colour_tail(w, round);
            if (!grid_barrier(w)) return;
            break;
        }
        if (round >= kMaxColours - kFirstFitColours) {
            /* cannot happen for rounds bounded by the maximum body degree; keep the kernel finite */
            for (int k = gtid; k < n; k += gsize)
                if (w.cons_colour[k] < 0) w.cons_colour[k] = kMaxColours - 1;
            if (gtid == 0) atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_COLOUR_OVERFLOW);
            break;
        }
        unsigned long long* offer = w.b_cmin + (size_t)(round & 1) * 2 * bc;
        unsigned long long* stale = w.b_cmin + (size_t)((round + 1) & 1) * 2 * bc;
        /* A: each uncoloured constraint offers its priority to its dynamic bodies */
        for (int k = gtid; k < n; k += gsize) {
            const int2 bd = w.c.body[w.cons_contact[k]];
            const size_t cm = w.cons_part[k] < 0 ? bc : 0;
            if (round > 0) {
                stale[cm + bd.x] = kNone;
                stale[cm + bd.y] = kNone;
            }
            if (w.cons_colour[k] >= 0) continue;
            const unsigned long long key = ((unsigned long long)hash32((uint32_t)k) << 32) | (uint32_t)k;
            if (is_dynamic(w.b_flags[bd.x])) atomicMin(&offer[cm + bd.x], key);
            if (is_dynamic(w.b_flags[bd.y])) atomicMin(&offer[cm + bd.y], key);
        }
        if (gtid == 0) w.cnt[CNT_UNCOLOURED + (round & 1)] = 0;
        if (!grid_barrier(w)) return;
        /* B: local minima take the lowest colour free at both bodies */
        for (int k = gtid; k < n; k += gsize) {
            if (w.cons_colour[k] >= 0) continue;
            const int2 bd = w.c.body[w.cons_contact[k]];
            const size_t cm = w.cons_part[k] < 0 ? bc : 0;
            const unsigned long long key = ((unsigned long long)hash32((uint32_t)k) << 32) | (uint32_t)k;
            const bool da = is_dynamic(w.b_flags[bd.x]), db = is_dynamic(w.b_flags[bd.y]);
            const bool winA = !da || offer[cm + bd.x] == key;
            const bool winB = !db || offer[cm + bd.y] == key;
            if (winA && winB) {
                const unsigned long long used =
                    (da ? w.b_cmask[cm + bd.x] : 0ull) | (db ? w.b_cmask[cm + bd.y] : 0ull);
                int colour;
                if (~used != 0ull) {
                    colour = __ffsll((long long)~used) - 1;
                    const unsigned long long bit = 1ull << colour;
                    if (da) w.b_cmask[cm + bd.x] |= bit;
                    if (db) w.b_cmask[cm + bd.y] |= bit;
                } else {
                    colour = kFirstFitColours + round;
                    if (colour >= kMaxColours) {
                        colour = kMaxColours - 1;
                        atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_COLOUR_OVERFLOW);
                    }
                }
                w.cons_colour[k] = colour;
            } else {
                agg_increment(&w.cnt[CNT_UNCOLOURED + (round & 1)]);
            }
        }
        ++round;
        if (!grid_barrier(w)) return;
    }
    if (gtid == 0 && w.cnt[CNT_TAIL] == 0) w.cnt[CNT_ROUNDS] = round;
    /* histogram rows: part p's interior colours are row p, the boundary colours row P */
    for (int k = gtid; k < n; k += gsize) {
        const int part = w.cons_part[k];
        atomicAdd(&w.col_hist[(part < 0 ? P : part) * kMaxColours + w.cons_colour[k]], 1);
    }
    if (!grid_barrier(w)) return;
    for (int r = blockIdx.x; r <= P; r += gridDim.x) {
        int tot;
        block_scan_excl(w.col_hist[r * kMaxColours + threadIdx.x], &tot);
        if (threadIdx.x == 0) w.part_tot[r] = tot;
    }
    if (!grid_barrier(w)) return;
    /* dense offsets of each row's non-empty colours; the histogram becomes the slot cursors */
    for (int r = blockIdx.x; r <= P; r += gridDim.x) {
        int part_sum = 0;
        for (int q = threadIdx.x; q < r; q += blockDim.x) part_sum += w.part_tot[q];
        int base;
        block_scan_excl(part_sum, &base);
        const int cnt = w.col_hist[r * kMaxColours + threadIdx.x];
        int tot, ndense;
        const int excl = block_scan_excl(cnt, &tot);
        const int dense = block_scan_excl(cnt > 0 ? 1 : 0, &ndense);
        int* out = r < P ? w.part_off + (size_t)r * (kMaxColours + 1) : w.col_off;
        if (cnt > 0) out[dense] = base + excl;
        w.col_hist[r * kMaxColours + threadIdx.x] = base + excl;
        if (threadIdx.x == 0) {
            out[ndense] = base + tot;
            if (r < P) {
                w.part_ncol[r] = ndense;
            } else {
                w.cnt[CNT_COLOURS] = ndense;
                w.cnt[CNT_INTERIOR] = base;
                w.cnt[CNT_PARTS] = P;
                if (rebalance) {
                    /* rank starts ascending: part 0 from rank 0, an empty part as wide as nothing */
                    int next = nf;
                    for (int q = P - 1; q > 0; --q) {
                        if (w.part_rbeg[q] == INT_MAX) w.part_rbeg[q] = next;
                        else next = w.part_rbeg[q];
                    }
                    w.part_rbeg[0] = 0;
                }
            }
        }
    }
    if (!grid_barrier(w)) return;
    const uint32_t next = (stamp + 1u) & kStampMask;
    for (int k = gtid; k < n; k += gsize) {
        const int c = w.cons_colour[k];
        const int ci = w.cons_contact[k];
        const int part = w.cons_part[k];
        const int slot = atomicAdd(&w.col_hist[(part < 0 ? P : part) * kMaxColours + c], 1);
        /* keep first-fit colours for the next colouring (the per-round overflow colours are not
         * kept: a later round could hand the same one to a neighbour) */
        w.c.mids[ci].w = (c < kFirstFitColours && next != 0u)
                             ? ((next << 7) | ((part < 0 ? 1u : 0u) << 6) | (uint32_t)c) : 0u;
        if (slot < 0 || slot >= n) continue;  /* cannot happen with consistent offsets */
        w.s_contact[slot] = ci;
        w.s_cons[slot] = k;
    }
    if (gtid == 0) w.cnt[CNT_COLOURINGS] = (int)next;
}

/* ---------------- solver (cooperative) ---------------- */
__device__ __forceinline__ V2 v2of(float x, float y) { return mk(x, y); }

/* B2contactSolver::new + initialize_velocity_constraints for one slot (make_constraint on the
 * world's arrays) */
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
    ConstraintIn in;
    in.mat = mat;
    in.geo = geo;
    in.pts = pts;
    in.imp = make_float4(ni0, ti0, ni1, ti1);
    in.mtype = mtype;
    in.count = count;
    in.ia = bd.x;
    in.ib = bd.y;
    in.flags = (is_dynamic(fa) ? 1 : 0) | (is_dynamic(fb) ? 2 : 0);
    in.mA = mA;
    in.iA = iA;
    in.mB = mB;
    in.iB = iB;
    in.rA = rA;
    in.rB = rB;
    in.lcA = lcA;
    in.lcB = lcB;
    in.cA = v2of(pA.x, pA.y);
    in.cB = v2of(pB.x, pB.y);
    in.vA = v2of(vA4.x, vA4.y);
    in.vB = v2of(vB4.x, vB4.y);
    in.wA = vA4.z;
    in.wB = vB4.z;
    /* xf.q = rot(angle): the bodies' transforms hold exactly that rotation of their current angles
     * (written from the same angle by the last copy-back, set_transform or creation), so it is
     * read instead of evaluating sin/cos again for every constraint */
    const float4 xa4 = w.b_xf[bd.x], xb4 = w.b_xf[bd.y];
    in.qA.s = xa4.z;
    in.qA.c = xa4.w;
    in.qB.s = xb4.z;
    in.qB.c = xb4.w;
    VelSlot vs;
    PosSlot ps;
    make_constraint(in, vs, ps);
    w.vc_idx[k] = vs.idx;
    w.vc_inv[k] = vs.inv;
    w.vc_nf[k] = vs.nf;
    w.vc_r0[k] = vs.r0;
    w.vc_r1[k] = vs.r1;
    w.vc_m0[k] = vs.m0;
    w.vc_m1[k] = vs.m1;
    w.vc_imp[k] = vs.imp;
    w.vc_k[k] = vs.k;
    w.pc_lp[k] = ps.lp;
    w.pc_geo[k] = ps.geo;
    w.pc_lc[k] = ps.lc;
    w.pc_inv[k] = ps.inv;
    w.pc_meta[k] = ps.meta;
    w.vc_island[k] = w.cons_island[w.s_cons[k]];
    w.s_fix[k] = fx;
}

__device__ __forceinline__ VelSlot vel_slot(const DevWorld& w, int k) {
    VelSlot s;
    s.idx = w.vc_idx[k];
    s.inv = w.vc_inv[k];
    s.nf = w.vc_nf[k];
    s.imp = w.vc_imp[k];
    s.r0 = w.vc_r0[k];
    s.r1 = w.vc_r1[k];
    s.m0 = w.vc_m0[k];
    s.m1 = w.vc_m1[k];
    s.k = w.vc_k[k];
    return s;
}

__device__ __forceinline__ PosSlot pos_slot(const DevWorld& w, int k) {
    PosSlot s;
    s.idx = w.vc_idx[k];
    s.lp = w.pc_lp[k];
    s.geo = w.pc_geo[k];
    s.lc = w.pc_lc[k];
    s.inv = w.pc_inv[k];
    s.meta = w.pc_meta[k];
    s.island = w.vc_island[k];
    s.pad[0] = s.pad[1] = s.pad[2] = 0;  /* pad[0]: the island's early-exit flag (part-local solve) */
    return s;
}

/* the slot routines on the global body arrays (slot order by colour) */
__device__ __forceinline__ void warm_slot(const DevWorld& w, int k) {
    const VelSlot sl = vel_slot(w, k);
    float4 va = w.b_vel[sl.idx.x], vb = w.b_vel[sl.idx.y];
    warm_math(sl, va, vb);
    if (sl.idx.w & 1) w.b_vel[sl.idx.x] = va;
    if (sl.idx.w & 2) w.b_vel[sl.idx.y] = vb;
}

__device__ __forceinline__ void solve_velocity_slot(const DevWorld& w, int k) {
    const VelSlot sl = vel_slot(w, k);
    float4 va = w.b_vel[sl.idx.x], vb = w.b_vel[sl.idx.y];
    float4 imp = sl.imp;
    solve_velocity_math(sl, imp, va, vb);
    w.vc_imp[k] = imp;
    if (sl.idx.w & 1) w.b_vel[sl.idx.x] = va;
    if (sl.idx.w & 2) w.b_vel[sl.idx.y] = vb;
}

__device__ __forceinline__ float solve_position_slot(const DevWorld& w, int k) {
    const PosSlot sl = pos_slot(w, k);
    float4 pa = w.b_pos[sl.idx.x], pb = w.b_pos[sl.idx.y];
    const float ms = solve_position_math(sl, pa, pb);
    if (sl.idx.w & 1) w.b_pos[sl.idx.x] = pa;
    if (sl.idx.w & 2) w.b_pos[sl.idx.y] = pb;
    return ms;
}

/* ---------------- part-local solve ----------------
 * Block p owns part p: a range of the constraint bodies in Morton-rank order (ranges of equal
 * constraint work, set by the colouring). It caches their velocities (then positions) and its
 * interior constraint slots in shared memory, sweeps its interior colours separated by
 * __syncthreads, writes the bodies back, and the boundary colours follow grid-wide. A body or slot
 * that does not fit the cache is read and written in global memory by the same block, which alone
 * touches it in the interior phase. */
struct PartCtx {
    int cbeg;          /* the part's first entry of cache_body */
    int nloc;          /* bodies cached (body[] entries) */
    int ibeg;          /* first interior slot */
    int ncol;          /* non-empty interior colours */
    int cap_vel;       /* interior slots cached as VelSlot */
    int cap_pos;       /* interior slots cached as PosSlot */
    const int* off;    /* shared: offsets of the part's colours */
    float4* state;     /* shared: cached velocities or positions */
    int* body;         /* shared: the cached bodies */
    void* slots;       /* shared: VelSlot[cap_vel] or PosSlot[cap_pos] */
    void* bslots;      /* shared: this block's boundary slots, VelSlot or PosSlot[kBndSlots] */
    const int* bco;    /* shared: boundary colour offsets */
    const int* boff;   /* shared: per boundary colour, this block's first entry of bslots */
};

/* Boundary slots cached per block: each boundary colour is split evenly over the blocks, and a
 * block keeps its share of every colour (with global body indices) in shared memory. */
constexpr int kBndSlots = 128;
constexpr int kBndBytes = kBndSlots * (int)sizeof(VelSlot);

__device__ __forceinline__ void bnd_range(const PartCtx& pc, int c, int* lo, int* hi) {
    const int len = pc.bco[c + 1] - pc.bco[c];
    *lo = (int)((long long)len * blockIdx.x / gridDim.x);
    *hi = (int)((long long)len * (blockIdx.x + 1) / gridDim.x);
}

/* whether an island stopped before position iteration `it` (some earlier iteration ended with
 * min separation >= -3 slop) */
__device__ __forceinline__ bool island_done(const DevWorld& w, int isl, int it, float tol) {
    bool done = false;
    for (int q = 0; q < it && !done; ++q) done = __uint_as_float(w.isl_minsep[(size_t)q * w.body_cap + isl]) <= tol;
    return done;
}

/* one boundary colour of the warm start or a velocity iteration, this block's share; `last`: the
 * final velocity sweep, whose impulses go to global memory for store_impulses */
__device__ void bnd_vel_sweep(const DevWorld& w, const PartCtx& pc, int c, bool warm, bool last) {
    int lo, hi;
    bnd_range(pc, c, &lo, &hi);
    VelSlot* bs = (VelSlot*)pc.bslots;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int k = pc.bco[c] + i, j = pc.boff[c] + i - lo;
        const bool cached = j < kBndSlots;
        const VelSlot sl = cached ? bs[j] : vel_slot(w, k);
        float4 va = w.b_vel[sl.idx.x], vb = w.b_vel[sl.idx.y];
        if (warm) {
            warm_math(sl, va, vb);
        } else {
            float4 imp = sl.imp;
            solve_velocity_math(sl, imp, va, vb);
            if (cached && !last) bs[j].imp = imp;
            else w.vc_imp[k] = imp;
        }
        if (sl.idx.w & 1) w.b_vel[sl.idx.x] = va;
        if (sl.idx.w & 2) w.b_vel[sl.idx.y] = vb;
    }
}

/* one boundary colour of position iteration `it`, this block's share (cached slots carry their
 * island's early-exit flag in pad[0]) */
__device__ void bnd_pos_sweep(const DevWorld& w, const PartCtx& pc, int c, int it, uint32_t* cur, float tol) {
    int lo, hi;
    bnd_range(pc, c, &lo, &hi);
    const PosSlot* bs = (const PosSlot*)pc.bslots;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int k = pc.bco[c] + i, j = pc.boff[c] + i - lo;
        const bool cached = j < kBndSlots;
        const PosSlot sl = cached ? bs[j] : pos_slot(w, k);
        if (cached ? sl.pad[0] != 0 : island_done(w, sl.island, it, tol)) continue;
        float4 pa = w.b_pos[sl.idx.x], pb = w.b_pos[sl.idx.y];
        const float ms = solve_position_math(sl, pa, pb);
        if (sl.idx.w & 1) w.b_pos[sl.idx.x] = pa;
        if (sl.idx.w & 2) w.b_pos[sl.idx.y] = pb;
        agg_atomic_max(cur, sl.island, ms < 0.0f ? __float_as_uint(-ms) : 0u);
    }
}

/* early-exit flags of the block's cached interior and boundary position slots for iteration `it` */
__device__ void part_done_flags(const DevWorld& w, const PartCtx& pc, int nbnd, int it, float tol) {
    PosSlot* ps = (PosSlot*)pc.slots;
    PosSlot* bs = (PosSlot*)pc.bslots;
    for (int j = threadIdx.x; j < pc.cap_pos; j += blockDim.x) ps[j].pad[0] = island_done(w, ps[j].island, it, tol) ? 1 : 0;
    for (int j = threadIdx.x; j < nbnd; j += blockDim.x) bs[j].pad[0] = island_done(w, bs[j].island, it, tol) ? 1 : 0;
}

__device__ __forceinline__ int body_code(const DevWorld& w, const PartCtx& pc, int b, bool dyn) {
    if (dyn) {
        const int l = w.b_cidx[b] - pc.cbeg;
        if (l >= 0 && l < pc.nloc && pc.body[l] == b) return l;
    }
    return -(b + 1);
}

__device__ __forceinline__ float4 ld_body(const float4* st, const float4* glob, int code) {
    return code >= 0 ? st[code] : glob[-code - 1];
}

__device__ __forceinline__ void st_body(float4* st, float4* glob, int code, float4 v) {
    if (code >= 0) st[code] = v;
    else glob[-code - 1] = v;
}

__device__ __forceinline__ VelSlot part_vel_slot(const DevWorld& w, const PartCtx& pc, int k) {
    VelSlot sl = vel_slot(w, k);
    sl.idx.x = body_code(w, pc, sl.idx.x, (sl.idx.w & 1) != 0);
    sl.idx.y = body_code(w, pc, sl.idx.y, (sl.idx.w & 2) != 0);
    return sl;
}

__device__ __forceinline__ PosSlot part_pos_slot(const DevWorld& w, const PartCtx& pc, int k) {
    PosSlot sl = pos_slot(w, k);
    sl.idx.x = body_code(w, pc, sl.idx.x, (sl.idx.w & 1) != 0);
    sl.idx.y = body_code(w, pc, sl.idx.y, (sl.idx.w & 2) != 0);
    return sl;
}

/* a slot outside the block's cache, with the body codes its block wrote at the step's start (a load
 * beside the slot's own instead of a lookup after it) */
__device__ __forceinline__ VelSlot coded_vel_slot(const DevWorld& w, int k) {
    VelSlot sl = vel_slot(w, k);
    const int2 code = w.vc_code[k];
    sl.idx.x = code.x;
    sl.idx.y = code.y;
    return sl;
}
__device__ __forceinline__ PosSlot coded_pos_slot(const DevWorld& w, int k) {
    PosSlot sl = pos_slot(w, k);
    const int2 code = w.vc_code[k];
    sl.idx.x = code.x;
    sl.idx.y = code.y;
    return sl;
}

/* one velocity constraint of a part (warm start or a velocity iteration) on bodies va, vb */
__device__ __forceinline__ void part_vel_solve(const VelSlot& sl, bool warm, float4& va, float4& vb, float4& imp) {
    imp = sl.imp;
    if (warm) warm_math(sl, va, vb);
    else solve_velocity_math(sl, imp, va, vb);
}

/* the part's interior colours (warm start or one velocity iteration). Slots in shared memory come
 * first; the rest are read from global memory two per thread at a time: both slots' loads, then
 * both pairs of bodies, are in flight together (constraints of one colour share no body, so the
 * two are independent and their order is immaterial). */
__device__ void part_vel_sweeps(const DevWorld& w, const PartCtx& pc, bool warm) {
    VelSlot* vs = (VelSlot*)pc.slots;
    for (int c = 0; c < pc.ncol; ++c) {
        const int beg = pc.off[c], end = pc.off[c + 1];
        const int kc = max(beg, min(end, pc.ibeg + pc.cap_vel));  /* [beg, kc) cached */
        for (int k = beg + threadIdx.x; k < kc; k += blockDim.x) {
            const int j = k - pc.ibeg;
            const VelSlot sl = vs[j];
            float4 va = ld_body(pc.state, w.b_vel, sl.idx.x), vb = ld_body(pc.state, w.b_vel, sl.idx.y);
            float4 imp;
            part_vel_solve(sl, warm, va, vb, imp);
            if (!warm) vs[j].imp = imp;
            if (sl.idx.w & 1) st_body(pc.state, w.b_vel, sl.idx.x, va);
            if (sl.idx.w & 2) st_body(pc.state, w.b_vel, sl.idx.y, vb);
        }
        for (int k0 = kc + threadIdx.x; k0 < end; k0 += 2 * blockDim.x) {
            const int k1 = k0 + (int)blockDim.x;
            const bool two = k1 < end;
            const VelSlot s0 = coded_vel_slot(w, k0);
            const VelSlot s1 = coded_vel_slot(w, two ? k1 : k0);
            float4 va0 = ld_body(pc.state, w.b_vel, s0.idx.x), vb0 = ld_body(pc.state, w.b_vel, s0.idx.y);
            float4 va1 = ld_body(pc.state, w.b_vel, s1.idx.x), vb1 = ld_body(pc.state, w.b_vel, s1.idx.y);
            float4 imp0, imp1;
            part_vel_solve(s0, warm, va0, vb0, imp0);
            if (!warm) w.vc_imp[k0] = imp0;
            if (s0.idx.w & 1) st_body(pc.state, w.b_vel, s0.idx.x, va0);
            if (s0.idx.w & 2) st_body(pc.state, w.b_vel, s0.idx.y, vb0);
            if (two) {
                part_vel_solve(s1, warm, va1, vb1, imp1);
                if (!warm) w.vc_imp[k1] = imp1;
                if (s1.idx.w & 1) st_body(pc.state, w.b_vel, s1.idx.x, va1);
                if (s1.idx.w & 2) st_body(pc.state, w.b_vel, s1.idx.y, vb1);
            }
        }
        __syncthreads();
    }
}

/* the part's interior colours of position iteration `it` (per-island early exit as in k_solve) */
__device__ void part_pos_sweeps(const DevWorld& w, const PartCtx& pc, int it, uint32_t* cur, float tol) {
    const PosSlot* ps = (const PosSlot*)pc.slots;
    for (int c = 0; c < pc.ncol; ++c) {
        const int beg = pc.off[c], end = pc.off[c + 1];
        const int kc = max(beg, min(end, pc.ibeg + pc.cap_pos));  /* [beg, kc) cached */
        for (int k = beg + threadIdx.x; k < kc; k += blockDim.x) {
            const PosSlot sl = ps[k - pc.ibeg];
            if (sl.pad[0] != 0) continue;
            float4 pa = ld_body(pc.state, w.b_pos, sl.idx.x), pb = ld_body(pc.state, w.b_pos, sl.idx.y);
            const float ms = solve_position_math(sl, pa, pb);
            if (sl.idx.w & 1) st_body(pc.state, w.b_pos, sl.idx.x, pa);
            if (sl.idx.w & 2) st_body(pc.state, w.b_pos, sl.idx.y, pb);
            agg_atomic_max(cur, sl.island, ms < 0.0f ? __float_as_uint(-ms) : 0u);
        }
        /* slots in global memory two per thread at a time, as in part_vel_sweeps */
        for (int k0 = kc + threadIdx.x; k0 < end; k0 += 2 * blockDim.x) {
            const int k1 = k0 + (int)blockDim.x;
            const bool two = k1 < end;
            const PosSlot s0 = coded_pos_slot(w, k0);
            const PosSlot s1 = coded_pos_slot(w, two ? k1 : k0);
            const bool run0 = !island_done(w, s0.island, it, tol);
            const bool run1 = two && !island_done(w, s1.island, it, tol);
            float4 pa0 = ld_body(pc.state, w.b_pos, s0.idx.x), pb0 = ld_body(pc.state, w.b_pos, s0.idx.y);
            float4 pa1 = ld_body(pc.state, w.b_pos, s1.idx.x), pb1 = ld_body(pc.state, w.b_pos, s1.idx.y);
            float ms0 = 0.0f, ms1 = 0.0f;
            if (run0) {
                ms0 = solve_position_math(s0, pa0, pb0);
                if (s0.idx.w & 1) st_body(pc.state, w.b_pos, s0.idx.x, pa0);
                if (s0.idx.w & 2) st_body(pc.state, w.b_pos, s0.idx.y, pb0);
            }
            if (run1) {
                ms1 = solve_position_math(s1, pa1, pb1);
                if (s1.idx.w & 1) st_body(pc.state, w.b_pos, s1.idx.x, pa1);
                if (s1.idx.w & 2) st_body(pc.state, w.b_pos, s1.idx.y, pb1);
            }
            agg_atomic_max(cur, s0.island, ms0 < 0.0f ? __float_as_uint(-ms0) : 0u);
            agg_atomic_max(cur, s1.island, ms1 < 0.0f ? __float_as_uint(-ms1) : 0u);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void part_store(const PartCtx& pc, float4* glob) {
    for (int l = threadIdx.x; l < pc.nloc; l += blockDim.x) {
        const int b = pc.body[l];
        if (b >= 0) glob[b] = pc.state[l];
    }
}

__device__ __forceinline__ void part_load(const PartCtx& pc, const float4* glob) {
    for (int l = threadIdx.x; l < pc.nloc; l += blockDim.x) {
        const int b = pc.body[l];
        if (b >= 0) pc.state[l] = glob[b];
    }
}

/* Islands and the constraint list in one cooperative launch, its passes separated by grid barriers:
 * reset, union over the constraints and joints (B2world::solve's DFS, private/dynamics/
 * b2_world.rs:375-491, as connected components), each body's root and its island's awake flag,
 * the solved bodies' flags, then the constraint list in contact order (each block counts its chunk
 * of the table, the chunks' counts give each block its offset, and a block scan places the block's
 * constraints). */
__global__ void __launch_bounds__(kBlock) k_islands(DevWorld w, int allow_sleep) {
    B2G_RETURN_IF_ABORTED(w);
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    const int nb = w.n_bodies;
    for (int b = gtid; b < nb; b += gsize) {
        w.b_island[b] = b;
        w.isl_minsep[w.body_cap + b] = 0u;  /* "island has an awake member" */
        w.b_flags[b] &= ~BF_ISLAND;
        if (allow_sleep) w.isl_sleep[b] = kMaxFloat;
    }
    if (!grid_barrier(w)) return;
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = gtid; i < n; i += gsize) {
        if (!contact_is_constraint(w.c.flags[i])) continue;
        const int2 bd = w.c.body[i];
        if (is_static(w.b_flags[bd.x]) || is_static(w.b_flags[bd.y])) continue;
        uf_union(w.b_island, bd.x, bd.y);
    }
    for (int j = gtid; j < w.n_joints; j += gsize) {
        const int2 bd = w.j_body[j];
        const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
        if (is_static(fa) || is_static(fb) || !(fa & BF_ENABLED) || !(fb & BF_ENABLED)) continue;
        uf_union(w.b_island, bd.x, bd.y);
    }
    if (!grid_barrier(w)) return;
    for (int b = gtid; b < nb; b += gsize) {
        const int r = uf_find(w.b_island, b);
        const uint32_t f = w.b_flags[b];
        agg_atomic_or(w.isl_minsep + w.body_cap, r, ((f & BF_AWAKE) && (f & BF_ENABLED) && !is_static(f)) ? 1u : 0u);
    }
    if (!grid_barrier(w)) return;
    for (int b = gtid; b < nb; b += gsize) {
        int r = w.b_island[b];
        r = w.b_island[r];
        while (w.b_island[r] != r) r = w.b_island[r];
        w.b_island[b] = r;
        const uint32_t f = w.b_flags[b];
        if (!is_static(f) && (f & BF_ENABLED) && w.isl_minsep[w.body_cap + r]) w.b_flags[b] = f | BF_AWAKE | BF_ISLAND;
    }
    if (!grid_barrier(w)) return;
    /* the constraint list: this block's chunk of the contact table */
    const int chunk = (n + (int)gridDim.x - 1) / (int)gridDim.x;
    const int c0 = min(n, (int)blockIdx.x * chunk), c1 = min(n, c0 + chunk);
    auto selected = [&](int i) {
        if (!contact_is_constraint(w.c.flags[i])) return 0;
        const int2 bd = w.c.body[i];
        return ((w.b_flags[bd.x] & BF_ISLAND) || (w.b_flags[bd.y] & BF_ISLAND)) ? 1 : 0;
    };
    int mine = 0;
    for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) mine += selected(i);
    int block_total;
    block_scan_excl(mine, &block_total);
    if (threadIdx.x == 0) w.blk_tot[blockIdx.x] = (unsigned long long)block_total;
    if (!grid_barrier(w)) return;
    int before_part = 0, all_part = 0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
        const int t = (int)w.blk_tot[q];
        if (q < (int)blockIdx.x) before_part += t;
        all_part += t;
    }
    int before, all;
    block_scan_excl(before_part, &before);
    block_scan_excl(all_part, &all);
    int carry = 0;
    for (int base = c0; base < c1; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int sel = i < c1 ? selected(i) : 0;
        int tot;
        const int ex = block_scan_excl(sel, &tot);
        if (sel) {
            const int k = before + carry + ex;
            if (k < w.cons_cap) {
                const int2 bd = w.c.body[i];
                const int b = is_static(w.b_flags[bd.x]) ? bd.y : bd.x;
                w.cons_contact[k] = i;
                w.cons_island[k] = w.b_island[b];
            } else {
                atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_CONTACT_OVERFLOW);
            }
        }
        carry += tot;
    }
    if (gtid == 0) w.cnt[CNT_CONS] = min(all, w.cons_cap);
}

/* k_solve runs 256 or 512 threads per block (cfg_solver_block); nothing in it depends on which */
constexpr int kSolveMaxBlock = 512;

__global__ void __launch_bounds__(kSolveMaxBlock) k_solve(DevWorld w, StepParams sp) {
    B2G_RETURN_IF_ABORTED(w);
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
    const int interior = w.cnt[CNT_INTERIOR];
    const bool parts = interior > 0;
    const int nparts = w.cnt[CNT_PARTS];
    if (parts && (nparts <= 0 || nparts > (int)gridDim.x)) {  /* the same for every block: all return */
        if (gtid == 0) atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_PART_MISMATCH);
        return;
    }
    extern __shared__ float4 s_part[];
    __shared__ int s_off[kMaxColours + 1];
    __shared__ int s_bco[kMaxColours + 1];
    __shared__ int s_boff[kMaxColours + 1];
    PartCtx pc{};
    if (parts) {
        /* this block's part: its rank range, colour offsets and shared-memory caches (blocks
         * past the part count own none and only join the boundary sweeps) */
        const int p = blockIdx.x;
        const bool owner = p < nparts;
        pc.cbeg = owner ? w.part_cbeg[p] : 0;
        pc.nloc = owner ? max(0, min(w.part_cend[p] - pc.cbeg, sp.part_bodies)) : 0;
        pc.ncol = owner ? w.part_ncol[p] : 0;
        for (int i = threadIdx.x; owner && i <= pc.ncol; i += blockDim.x)
            s_off[i] = w.part_off[(size_t)p * (kMaxColours + 1) + i];
        pc.off = s_off;
        pc.state = s_part;
        pc.body = (int*)(s_part + sp.part_bodies);
        pc.bslots = (void*)(s_part + sp.part_bodies + (sp.part_bodies + 3) / 4);
        pc.slots = (void*)((char*)pc.bslots + kBndBytes);
        pc.bco = s_bco;
        pc.boff = s_boff;
        for (int i = threadIdx.x; i <= ncol; i += blockDim.x) s_bco[i] = w.col_off[i];
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int c = 0; c < ncol; ++c) {
                int lo, hi;
                bnd_range(pc, c, &lo, &hi);
                s_boff[c] = acc;
                acc += hi - lo;
            }
            s_boff[ncol] = acc;
        }
        pc.ibeg = pc.ncol > 0 ? s_off[0] : 0;
        const int nint = pc.ncol > 0 ? s_off[pc.ncol] - pc.ibeg : 0;
        const int islot_bytes = max(0, sp.part_slot_bytes - kBndBytes);
        pc.cap_vel = min(nint, islot_bytes / (int)sizeof(VelSlot));
        pc.cap_pos = min(nint, islot_bytes / (int)sizeof(PosSlot));
        for (int l = threadIdx.x; l < pc.nloc; l += blockDim.x) {
            const int b = w.cache_body[pc.cbeg + l];
            pc.body[l] = b;
            pc.state[l] = w.b_vel[b];
        }
        __syncthreads();
        VelSlot* vs = (VelSlot*)pc.slots;
        for (int j = threadIdx.x; j < pc.cap_vel; j += blockDim.x) vs[j] = part_vel_slot(w, pc, pc.ibeg + j);
        /* the body codes of the slots read from global memory (the position sweeps' too: a PosSlot is
         * smaller, so no fewer of them are cached) */
        for (int j = pc.cap_vel + threadIdx.x; j < nint; j += blockDim.x) {
            const int4 idx = w.vc_idx[pc.ibeg + j];
            w.vc_code[pc.ibeg + j] = make_int2(body_code(w, pc, idx.x, (idx.w & 1) != 0),
                                               body_code(w, pc, idx.y, (idx.w & 2) != 0));
        }
        for (int c = 0; c < ncol; ++c) {
            int lo, hi;
            bnd_range(pc, c, &lo, &hi);
            for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
                const int j = s_boff[c] + i - lo;
                if (j < kBndSlots) ((VelSlot*)pc.bslots)[j] = vel_slot(w, s_bco[c] + i);
            }
        }
        __syncthreads();
        /* phases 2 and 3: the warm start and each velocity iteration sweep the interior colours
         * of every part, then the boundary colours grid-wide */
        const int nsweeps = (sp.warm ? 1 : 0) + sp.vi;
        for (int sw = 0; sw < nsweeps; ++sw) {
            const bool warm = sp.warm && sw == 0;
            const bool last = sw == nsweeps - 1;
            part_vel_sweeps(w, pc, warm);
            if (last)
                for (int j = threadIdx.x; j < pc.cap_vel; j += blockDim.x) w.vc_imp[pc.ibeg + j] = vs[j].imp;
            if (ncol > 0 || last) part_store(pc, w.b_vel);
            if (ncol > 0) {
                if (!grid_barrier(w)) return;
                for (int c = 0; c < ncol; ++c) {
                    bnd_vel_sweep(w, pc, c, warm, last);
                    if (!grid_barrier(w)) return;
                }
                if (!last) {
                    part_load(pc, w.b_vel);
                    __syncthreads();
                }
            } else if (last) {
                if (!grid_barrier(w)) return;
            }
        }
    } else {
        /* phase 2: warm start, colour by colour */
        if (sp.warm) {
            for (int c = 0; c < ncol; ++c) {
                const int beg = w.col_off[c], end = w.col_off[c + 1];
                for (int k = beg + gtid; k < end; k += gsize) warm_slot(w, k);
                if (!grid_barrier(w)) return;
            }
        }
        /* phase 2b: the joints' init_velocity_constraints (with their warm start) follow the
         * contacts' warm start, joint colour by joint colour (b2_island_private.rs:196-201) */
        for (int c = 0; c < w.n_jcolours; ++c) {
            for (int q = w.j_coff[c] + gtid; q < w.j_coff[c + 1]; q += gsize) {
                const int j = w.j_order[q];
                if (joint_island(w, j) >= 0) joint_init_velocity(w, sp, j);
            }
            if (!grid_barrier(w)) return;
        }
        /* phase 3: velocity iterations, joints before contacts (:205-215) */
        for (int it = 0; it < sp.vi; ++it) {
            for (int c = 0; c < w.n_jcolours; ++c) {
                for (int q = w.j_coff[c] + gtid; q < w.j_coff[c + 1]; q += gsize) {
                    const int j = w.j_order[q];
                    if (joint_island(w, j) >= 0) joint_solve_velocity(w, sp, j);
                }
                if (!grid_barrier(w)) return;
            }
            for (int c = 0; c < ncol; ++c) {
                const int beg = w.col_off[c], end = w.col_off[c + 1];
                for (int k = beg + gtid; k < end; k += gsize) solve_velocity_slot(w, k);
                if (!grid_barrier(w)) return;
            }
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
    if (parts && sp.pi > 0) {
        for (int l = threadIdx.x; l < pc.nloc; l += blockDim.x) {
            const int b = pc.body[l];
            if (b >= 0) pc.state[l] = w.b_pos[b];
        }
        PosSlot* ps = (PosSlot*)pc.slots;
        for (int j = threadIdx.x; j < pc.cap_pos; j += blockDim.x) ps[j] = part_pos_slot(w, pc, pc.ibeg + j);
        for (int c = 0; c < ncol; ++c) {
            int lo, hi;
            bnd_range(pc, c, &lo, &hi);
            for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
                const int j = s_boff[c] + i - lo;
                if (j < kBndSlots) ((PosSlot*)pc.bslots)[j] = pos_slot(w, s_bco[c] + i);
            }
        }
        __syncthreads();
    }
    const int nbnd = parts ? min(s_boff[ncol], kBndSlots) : 0;
    for (int it = 0; it < sp.pi; ++it) {
        uint32_t* cur = w.isl_minsep + (size_t)it * w.body_cap;
        if (parts) {
            /* the interior colours, then a barrier: islands span parts, and the next iteration's
             * early exit reads this iteration's buffer. Without boundary constraints (a batch cut at
             * world boundaries) no island spans two parts: each part's islands are written by its
             * own block alone, so the iterations need no grid barrier until the positions go back. */
            if (it > 0) {
                part_done_flags(w, pc, nbnd, it, tol);
                __syncthreads();
            }
            part_pos_sweeps(w, pc, it, cur, tol);
            if (ncol > 0) {
                part_store(pc, w.b_pos);
                if (!grid_barrier(w)) return;
                for (int c = 0; c < ncol; ++c) {
                    bnd_pos_sweep(w, pc, c, it, cur, tol);
                    if (!grid_barrier(w)) return;
                }
                if (it < sp.pi - 1) {
                    part_load(pc, w.b_pos);
                    __syncthreads();
                }
            } else if (it == sp.pi - 1) {
                part_store(pc, w.b_pos);
                if (!grid_barrier(w)) return;
            }
            continue;
        }
        for (int c = 0; c < ncol; ++c) {
            const int beg = w.col_off[c], end = w.col_off[c + 1];
            for (int k = beg + gtid; k < end; k += gsize) {
                const int isl = w.vc_island[k];
                bool done = false;
                for (int j = 0; j < it && !done; ++j)
                    done = __uint_as_float(w.isl_minsep[(size_t)j * w.body_cap + isl]) <= tol;
                if (done) continue;
                const float ms = solve_position_slot(w, k);
                agg_atomic_max(cur, isl, ms < 0.0f ? __float_as_uint(-ms) : 0u);
            }
            if (!grid_barrier(w)) return;
        }
        /* the joints after the contacts; a joint out of its slop keeps its island going
         * (contacts_okay && joints_okay, b2_island_private.rs:257-274) */
        for (int c = 0; c < w.n_jcolours; ++c) {
            for (int q = w.j_coff[c] + gtid; q < w.j_coff[c + 1]; q += gsize) {
                const int j = w.j_order[q];
                const int isl = joint_island(w, j);
                if (isl < 0) continue;
                bool done = false;
                for (int jt = 0; jt < it && !done; ++jt)
                    done = __uint_as_float(w.isl_minsep[(size_t)jt * w.body_cap + isl]) <= tol;
                if (done) continue;
                if (!joint_solve_position(w, j)) atomicMax(&cur[isl], __float_as_uint(kMaxFloat));
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
                agg_atomic_min((unsigned*)w.isl_sleep, w.b_island[b], __float_as_uint(st));
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
    /* phase 6b: synchronize fixtures (private/dynamics/b2_body.rs:455-475); the proxies moved are
     * counted for the broadphase's rebuild decision */
    unsigned moved = 0;
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
        if (sync_fixture(w, f, xf1, xf2)) ++moved;
    }
    moved = __reduce_add_sync(0xffffffffu, moved);
    if ((threadIdx.x & 31) == 0 && moved) atomicAdd(&w.cnt[CNT_BP_MOVED], (int)moved);
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
    B2G_RETURN_IF_ABORTED(w);
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

/* k_islands runs one block per SM for a world of up to 64k bodies and more blocks per SM for larger
 * ones (up to what can be co-resident): its passes stride over all bodies and contacts, so a large
 * batch wants more threads in flight, while a small world wants the shortest grid barriers. */
void launch_islands_and_constraints(const DevWorld& w, const StepParams& sp, cudaStream_t s) {
    if (w.n_bodies > 0) {
        static int resident = 0;
        if (!resident) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, (const void*)k_islands, kBlock, 0);
            resident = std::max(1, std::min(resident, 8));
        }
        const int per_sm = std::max(1, std::min(resident, w.n_bodies / 65536));
        DevWorld wc = w;
        int allow_sleep = sp.allow_sleep;
        void* args[] = {&wc, &allow_sleep};
        cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
        cudaLaunchCooperativeKernel((const void*)k_islands, dim3(w.num_sms * per_sm), dim3(kBlock), args, 0, s);
        B2G_LAUNCHED(1);
    }
}

/* Parts of the part-local solve: about one per 256 proxies, at most one per SM, whatever the
 * blocks per SM (so results do not depend on the launch configuration). A small world is one
 * part, solved by one block without grid barriers between its colours. */
int part_count(const DevWorld& w, int num_sms) {
    return std::max(1, std::min(std::min(num_sms, kMaxParts), w.n_fixtures / 256));
}

/* In one world the part-local solve pays off while a part's bodies and constraints fit its block's
 * shared memory; a larger world (thousands of proxies per SM) keeps the grid-wide colour sweeps,
 * which spread each colour over every thread of the GPU. A batch of worlds is cut at world
 * boundaries (no boundary colours, no grid barrier inside the sweeps), so it takes parts at any
 * size: what its cache does not hold a part's block reads in global memory. */
constexpr int kPartMaxProxiesPerSm = 2048;

bool use_parts(const DevWorld& w, int num_sms, bool allowed) {
    /* joints are solved grid-wide before each contact sweep, so a world with joints runs the
     * grid-wide colour schedule */
    return allowed && w.n_joints == 0 && w.n_fixtures > 0 &&
           (w.num_worlds > 1 || (long long)w.n_fixtures <= (long long)num_sms * kPartMaxProxiesPerSm);
}

void launch_colouring(const DevWorld& w, cudaStream_t s, int num_sms, bool parts) {
    /* more blocks per SM for large worlds (as k_islands): the colouring's passes stride over every
     * constraint and body */
    static int resident = 0;
    if (!resident) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, (const void*)k_colour, kBlock, 0);
        resident = std::max(1, std::min(resident, 8));
    }
    const int per_sm = std::max(w.cfg_coop_per_sm, std::min(resident, w.n_bodies / 65536));
    const int blocks = coop_blocks((const void*)k_colour, num_sms) * per_sm;
    DevWorld wc = w;
    int nparts = use_parts(w, num_sms, parts) ? part_count(w, num_sms) : 0;
    void* args[] = {&wc, &nparts};
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    cudaLaunchCooperativeKernel((const void*)k_colour, dim3(blocks), dim3(kBlock), args, 0, s);
    B2G_LAUNCHED(1);
}

/* Shared memory of the part-local solve per block: most of an SM's with one block per SM, half
 * of it with two; none with more (the part-local sweeps then work in global memory). There is
 * one part per SM. */
constexpr int kPartSmemOne = 200 * 1024;
constexpr int kPartSmemTwo = 96 * 1024;

int launch_solver(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms, bool parts) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute((const void*)k_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, kPartSmemOne);
        attr_set = true;
    }
    const int blocks = coop_blocks((const void*)k_solve, num_sms) * w.cfg_coop_per_sm;
    DevWorld wc = w;
    StepParams spc = sp;
    size_t smem = 0;
    spc.part_bodies = 0;
    spc.part_slot_bytes = 0;
    if (use_parts(w, num_sms, parts)) {
        const int budget = w.cfg_coop_per_sm == 1 ? kPartSmemOne : (w.cfg_coop_per_sm == 2 ? kPartSmemTwo : 0);
        /* a part holds at most ceil(n_fixtures / blocks) ranks; bodies take at most half */
        const int nb = (budget / 4 / 20) & ~3;  /* a quarter of it for bodies */
        const int body_bytes = (nb + nb / 4) * 16;
        spc.part_bodies = nb;
        spc.part_slot_bytes = std::max(0, budget - body_bytes);
        smem = (size_t)(budget > 0 ? body_bytes + spc.part_slot_bytes : 0);
    }
    void* args[] = {&wc, &spc};
    B2G_LAUNCHED(1);
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    const int threads = w.cfg_coop_per_sm == 1 && w.cfg_solver_block == kSolveMaxBlock ? kSolveMaxBlock : kBlock;
    return (int)cudaLaunchCooperativeKernel((const void*)k_solve, dim3(blocks), dim3(threads), args, smem, s);
}

void launch_set_transform(const DevWorld& w, int body, float px, float py, float angle, cudaStream_t s) {
    k_set_transform<<<grid_for(w.n_fixtures, kBlock, w.num_sms * 4), kBlock, 0, s>>>(w, body, px, py, angle); B2G_LAUNCHED(1);
}

void launch_clear_forces(const DevWorld& w, cudaStream_t s) {
    k_clear_forces<<<grid_for(w.n_bodies, kBlock, w.num_sms * 4), kBlock, 0, s>>>(w); B2G_LAUNCHED(1);
}

}  // namespace b2g
