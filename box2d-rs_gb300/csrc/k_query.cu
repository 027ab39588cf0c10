/*
 * k_query.cu — world queries on the step's LBVH: many AABB queries or ray casts in one launch.
 *
 * Reference: B2world::query_aabb and B2world::ray_cast (private/dynamics/b2_world.rs:969-1056)
 * over B2dynamicTree::query / ray_cast (src/b2_dynamic_tree.rs:239-347), with the fixtures' ray
 * casts B2circleShape (private/collision/b2_circle_shape.rs:26-59), B2polygonShape
 * (private/collision/b2_polygon_shape.rs:226-287) and B2edgeShape
 * (private/collision/b2_edge_shape.rs:39-102).
 *
 * One thread per query walks the hierarchy built by the last step's broadphase (fat AABBs as of
 * that step). A ray keeps the reference's clipping: every hit clips the segment to its fraction,
 * so the result is the closest hit; only the order in which equally distant fixtures are met can
 * differ from the reference's tree (the GPU keeps the first it meets).
 */
#include <climits>

#include "b2g_internal.h"

namespace b2g {
namespace {

constexpr int kBlock = 128;
constexpr int kStack = 64;

__device__ __forceinline__ bool aabb_overlap(const float4 a, const float4 b) {
    /* b2_test_overlap, src/b2_collision.rs:355-368 (closed boxes) */
    if (b.x - a.z > 0.0f || b.y - a.w > 0.0f) return false;
    if (a.x - b.z > 0.0f || a.y - b.w > 0.0f) return false;
    return true;
}

/* the separating-axis test of the tree ray cast: |dot(v, p1 - c)| - dot(|v|, h) > 0 separates */
__device__ __forceinline__ bool ray_box(const float4 box, const float4 seg, V2 p1, V2 v, V2 abs_v) {
    if (!aabb_overlap(box, seg)) return false;
    const V2 c = scale(0.5f, add(mk(box.x, box.y), mk(box.z, box.w)));
    const V2 h = scale(0.5f, sub(mk(box.z, box.w), mk(box.x, box.y)));
    const float separation = fabsf(dot(v, sub(p1, c))) - dot(abs_v, h);
    return !(separation > 0.0f);
}

__device__ bool shape_ray_cast(const ShapeRec& sh, const Xf& xf, V2 ip1, V2 ip2, float max_fraction, float* fraction,
                               V2* normal) {
    const int type = shape_type(sh);
    if (type == SHAPE_CIRCLE) {
        const V2 position = add(xf.p, mul(xf.q, sh.v[0]));
        const V2 s = sub(ip1, position);
        const float b = dot(s, s) - sh.radius * sh.radius;
        const V2 r = sub(ip2, ip1);
        const float c = dot(s, r);
        const float rr = dot(r, r);
        const float sigma = c * c - rr * b;
        if (sigma < 0.0f || rr < kEpsilon) return false;
        float a = -(c + fsqrt(sigma));
        if (0.0f <= a && a <= max_fraction * rr) {
            a = fdiv(a, rr);
            *fraction = a;
            V2 n = add(s, scale(a, r));
            normalize(n);
            *normal = n;
            return true;
        }
        return false;
    }
    const V2 p1 = mul_t(xf.q, sub(ip1, xf.p));
    const V2 p2 = mul_t(xf.q, sub(ip2, xf.p));
    const V2 d = sub(p2, p1);
    if (type == SHAPE_POLYGON) {
        /* the reference starts the entering bound at 0.032 (b2_polygon_shape.rs:239) */
        float lower = 0.032f, upper = max_fraction;
        int index = -1;
        const int count = shape_count(sh);
        for (int i = 0; i < count; ++i) {
            const float numerator = dot(sh.n[i], sub(sh.v[i], p1));
            const float denominator = dot(sh.n[i], d);
            if (denominator == 0.0f) {
                if (numerator < 0.0f) return false;
            } else if (denominator < 0.0f && numerator < lower * denominator) {
                lower = fdiv(numerator, denominator);
                index = i;
            } else if (denominator > 0.0f && numerator < upper * denominator) {
                upper = fdiv(numerator, denominator);
            }
            if (upper < lower) return false;
        }
        if (index >= 0) {
            *fraction = lower;
            *normal = mul(xf.q, sh.n[index]);
            return true;
        }
        return false;
    }
    /* edge: vertex1 = v[1], vertex2 = v[2] */
    const V2 v1 = sh.v[1], v2 = sh.v[2];
    const V2 e = sub(v2, v1);
    V2 nrm = mk(e.y, -e.x);
    normalize(nrm);
    const float numerator = dot(nrm, sub(v1, p1));
    if (shape_one_sided(sh) && numerator > 0.0f) return false;
    const float denominator = dot(nrm, d);
    if (denominator == 0.0f) return false;
    const float t = fdiv(numerator, denominator);
    if (t < 0.0f || max_fraction < t) return false;
    const V2 q = add(p1, scale(t, d));
    const V2 r = sub(v2, v1);
    const float rr = dot(r, r);
    if (rr == 0.0f) return false;
    const float sf = fdiv(dot(sub(q, v1), r), rr);
    if (sf < 0.0f || 1.0f < sf) return false;
    *fraction = t;
    *normal = numerator > 0.0f ? neg(mul(xf.q, nrm)) : mul(xf.q, nrm);
    return true;
}

__device__ __forceinline__ Xf body_xf(const DevWorld& w, int b) {
    const float4 x = w.b_xf[b];
    Xf xf;
    xf.p = mk(x.x, x.y);
    xf.q.s = x.z;
    xf.q.c = x.w;
    return xf;
}

/* one thread per ray: out_a = (fixture as int bits or -1, point x, point y, -),
 * out_b = (normal x, normal y, fraction, -) */
__global__ void __launch_bounds__(kBlock) k_ray_cast(DevWorld w, const float4* rays, const uint32_t* ray_world, int n,
                                                     float4* out_a, float4* out_b) {
    B2G_RETURN_IF_ABORTED(w);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 ray = rays[i];
        const V2 p1 = mk(ray.x, ray.y), p2 = mk(ray.z, ray.w);
        int hit = -1;
        V2 hit_point = mk(0.0f, 0.0f), hit_normal = mk(0.0f, 0.0f);
        float hit_fraction = 1.0f;
        const uint32_t wd = ray_world ? ray_world[i] : 0u;
        if (wd < (uint32_t)w.num_worlds) {
            V2 r = sub(p2, p1);
            normalize(r);
            const V2 v = mk(-1.0f * r.y, 1.0f * r.x);
            const V2 abs_v = mk(fabsf(v.x), fabsf(v.y));
            float max_fraction = 1.0f;
            auto seg_box = [&]() {
                const V2 t = add(p1, scale(max_fraction, sub(p2, p1)));
                const V2 lo = vmin(p1, t), hi = vmax(p1, t);
                return make_float4(lo.x, lo.y, hi.x, hi.y);
            };
            float4 seg = seg_box();
            auto leaf = [&](int p) {
                const int f = (int)w.bp_val[p];
                float fraction;
                V2 normal;
                if (shape_ray_cast(w.f_shape[f], body_xf(w, w.f_body[f]), p1, p2, max_fraction, &fraction, &normal)) {
                    hit = f;
                    hit_point = add(scale(1.0f - fraction, p1), scale(fraction, p2));
                    hit_normal = normal;
                    hit_fraction = fraction;
                    max_fraction = fraction;
                    seg = seg_box();
                }
            };
            /* the world's hierarchy, then the one of its large static proxies */
            for (int h = 0; h < 2; ++h) {
                const int root = w.bp_world_root[wd + (h ? (uint32_t)w.num_worlds : 0u)];
                if (root == INT_MIN) continue;
                if (root < 0) {  /* a hierarchy of one proxy */
                    if (ray_box(w.bp_leaf[~root], seg, p1, v, abs_v)) leaf(~root);
                    continue;
                }
                int stack[kStack];
                int top = 0;
                stack[top++] = root;
                while (top > 0) {
                    const int node = stack[--top];
                    const int2 ch = w.bp_node_child[node];
                    const float4 boxes[2] = {w.bp_node_b0[node], w.bp_node_b1[node]};
                    const int kids[2] = {ch.x, ch.y};
                    for (int c = 0; c < 2; ++c) {
                        if (!ray_box(boxes[c], seg, p1, v, abs_v)) continue;
                        if (kids[c] < 0) leaf(~kids[c]);
                        else if (top < kStack) stack[top++] = kids[c];
                        else atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_STACK_OVERFLOW);
                    }
                }
            }
        }
        out_a[i] = make_float4(__int_as_float(hit), hit_point.x, hit_point.y, 0.0f);
        out_b[i] = make_float4(hit_normal.x, hit_normal.y, hit_fraction, 0.0f);
    }
}

/* one thread per box: every fixture whose fat AABB overlaps it, as (query, fixture) pairs */
__global__ void __launch_bounds__(kBlock) k_query_aabb(DevWorld w, const float4* boxes, const uint32_t* box_world,
                                                       int n, uint2* out, int cap, int* count) {
    B2G_RETURN_IF_ABORTED(w);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 q = boxes[i];
        const uint32_t wd = box_world ? box_world[i] : 0u;
        if (wd >= (uint32_t)w.num_worlds) continue;
        auto emit = [&](int p) {
            const int slot = atomicAdd(count, 1);
            if (slot < cap) out[slot] = make_uint2((uint32_t)i, w.bp_val[p]);
        };
        for (int h = 0; h < 2; ++h) {
            const int root = w.bp_world_root[wd + (h ? (uint32_t)w.num_worlds : 0u)];
            if (root == INT_MIN) continue;
            if (root < 0) {
                if (aabb_overlap(w.bp_leaf[~root], q)) emit(~root);
                continue;
            }
            int stack[kStack];
            int top = 0;
            stack[top++] = root;
            while (top > 0) {
                const int node = stack[--top];
                const int2 ch = w.bp_node_child[node];
                const float4 bx[2] = {w.bp_node_b0[node], w.bp_node_b1[node]};
                const int kids[2] = {ch.x, ch.y};
                for (int c = 0; c < 2; ++c) {
                    if (!aabb_overlap(bx[c], q)) continue;
                    if (kids[c] < 0) emit(~kids[c]);
                    else if (top < kStack) stack[top++] = kids[c];
                    else atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_STACK_OVERFLOW);
                }
            }
        }
    }
}

}  // namespace

void launch_ray_cast(const DevWorld& w, const float4* rays, const uint32_t* ray_world, int n, float4* out_a,
                     float4* out_b, cudaStream_t s) {
    k_ray_cast<<<grid_for(n, kBlock, w.num_sms * 16), kBlock, 0, s>>>(w, rays, ray_world, n, out_a, out_b);
    B2G_LAUNCHED(1);
}

void launch_query_aabb(const DevWorld& w, const float4* boxes, const uint32_t* box_world, int n, uint2* out, int cap,
                       int* count, cudaStream_t s) {
    k_query_aabb<<<grid_for(n, kBlock, w.num_sms * 16), kBlock, 0, s>>>(w, boxes, box_world, n, out, cap, count);
    B2G_LAUNCHED(1);
}

}  // namespace b2g
