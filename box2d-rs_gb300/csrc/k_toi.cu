/*
 * k_toi.cu — time of impact of two moving shapes, many pairs per launch.
 *
 * Reference: b2_time_of_impact (private/collision/b2_time_of_impact.rs:191-463) with its
 * separation function (:10-189), the GJK distance b2_distance_fn
 * (private/collision/b2_distance.rs:331-440) with the simplex (:58-329) and the distance proxy
 * (:8-47, src/b2_distance.rs:12-130), and the sweep (src/b2_math.rs:764-787).
 *
 * One thread per pair runs the routines of b2g_toi.cuh (a long serial chain with little memory
 * traffic, so a pair stays in one thread's registers); results equal the host restatement bit for
 * bit.
 */
#include "b2g_toi.cuh"

namespace b2g {
namespace {

constexpr int kBlock = 128;

__global__ void __launch_bounds__(kBlock) k_time_of_impact(const ShapeRec* sa, const float4* swa, const ShapeRec* sb,
                                                           const float4* swb, const float* t_max, int n, int2* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        DistProxy pa, pb;
        make_proxy(sa[i], pa);
        make_proxy(sb[i], pb);
        Sweep a, b;
        {
            const float4 u = swa[2 * i], v = swa[2 * i + 1];
            a.lc = mk(u.x, u.y);
            a.c0 = mk(u.z, u.w);
            a.c = mk(v.x, v.y);
            a.a0 = v.z;
            a.a = v.w;
        }
        {
            const float4 u = swb[2 * i], v = swb[2 * i + 1];
            b.lc = mk(u.x, u.y);
            b.c0 = mk(u.z, u.w);
            b.c = mk(v.x, v.y);
            b.a0 = v.z;
            b.a = v.w;
        }
        int state;
        float t;
        time_of_impact(pa, a, pb, b, t_max ? t_max[i] : 1.0f, state, t);
        out[i] = make_int2(state, __float_as_int(t));
    }
}

}  // namespace

void launch_time_of_impact(const ShapeRec* sa, const float4* swa, const ShapeRec* sb, const float4* swb,
                           const float* t_max, int n, int2* out, cudaStream_t s) {
    k_time_of_impact<<<grid_for(n, kBlock, current_sm_count() * 16), kBlock, 0, s>>>(sa, swa, sb, swb, t_max, n, out);
    B2G_LAUNCHED(1);
}

}  // namespace b2g
