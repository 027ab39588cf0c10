/*
 * trig_check_gpu.cu — on the GPU: b2g_sincosf against b2g_sincosf_ref on every float with
 * 0 < |x| <= 8192, and the device results against the host's on a strided sample. Prints the
 * counts and exits non-zero on any mismatch.
 */
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "b2g_trig.h"

__global__ void k_check(unsigned top, unsigned long long* bad, unsigned long long* n) {
    unsigned long long lb = 0, ln = 0;
    for (unsigned u = 1u + blockIdx.x * blockDim.x + threadIdx.x; u <= top; u += gridDim.x * blockDim.x) {
        for (int sign = 0; sign < 2; ++sign) {
            const float x = sign ? -__uint_as_float(u) : __uint_as_float(u);
            float s1, c1, s2, c2;
            b2g_sincosf(x, &s1, &c1);
            b2g_sincosf_ref(x, &s2, &c2);
            lb += (__float_as_uint(s1) != __float_as_uint(s2)) || (__float_as_uint(c1) != __float_as_uint(c2));
            ++ln;
        }
    }
    atomicAdd(bad, lb);
    atomicAdd(n, ln);
}

__global__ void k_sample(const float* x, float* s, float* c, int m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) b2g_sincosf(x[i], &s[i], &c[i]);
}

int main() {
    float t = 8192.0f;
    unsigned top;
    std::memcpy(&top, &t, 4);
    unsigned long long *d_bad, *d_n, bad = 0, n = 0;
    cudaMalloc(&d_bad, 8);
    cudaMalloc(&d_n, 8);
    cudaMemset(d_bad, 0, 8);
    cudaMemset(d_n, 0, 8);
    k_check<<<152 * 8, 256>>>(top, d_bad, d_n);
    cudaMemcpy(&bad, d_bad, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(&n, d_n, 8, cudaMemcpyDeviceToHost);
    const int m = 1 << 22;
    std::vector<float> x(m), s(m), c(m);
    for (int i = 0; i < m; ++i) {
        unsigned u = 1u + (unsigned)((unsigned long long)i * (top - 1u) / (unsigned)m);
        std::memcpy(&x[i], &u, 4);
        if (i & 1) x[i] = -x[i];
    }
    float *dx, *ds, *dc;
    cudaMalloc(&dx, m * 4);
    cudaMalloc(&ds, m * 4);
    cudaMalloc(&dc, m * 4);
    cudaMemcpy(dx, x.data(), m * 4, cudaMemcpyHostToDevice);
    k_sample<<<(m + 255) / 256, 256>>>(dx, ds, dc, m);
    cudaMemcpy(s.data(), ds, m * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(c.data(), dc, m * 4, cudaMemcpyDeviceToHost);
    const cudaError_t err = cudaGetLastError();
    unsigned long long host_bad = 0;
    for (int i = 0; i < m; ++i) {
        float hs, hc;
        b2g_sincosf(x[i], &hs, &hc);
        host_bad += std::memcmp(&hs, &s[i], 4) != 0 || std::memcmp(&hc, &c[i], 4) != 0;
    }
    std::printf("device checked %llu mismatches %llu; device vs host sample %d mismatches %llu; %s\n", n, bad, m,
                host_bad, cudaGetErrorString(err));
    return (bad || host_bad || err != cudaSuccess || n == 0) ? 1 : 0;
}
