// GPU checks of the arithmetic helpers in asg_common.cuh that stand in for
// plain float operations (run by tests/test_gpu_helpers.py):
//   div   div_rn_by(a, L, 1/L) against __fdiv_rn(a, L) for every float a with
//         2^-20 <= |a| < 4096 and several box sides L;
//   x2    the packed f32x2 distance norm2_rn_x2 against the scalar norm2_rn on
//         seeded random point pairs.
// Prints one line per case with its mismatch count; exits 1 on any mismatch.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../asmooth_gb300/csrc/asg_common.cuh"

using namespace asg;

__global__ void k_div(uint32_t lo, uint32_t hi, float L, float rL, unsigned long long* bad)
{
    for (uint64_t b = lo + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < hi;
         b += (uint64_t)gridDim.x * blockDim.x)
        for (int sgn = 0; sgn < 2; ++sgn) {
            const float a = __uint_as_float((uint32_t)b | (sgn ? 0x80000000u : 0u));
            if (__float_as_uint(div_rn_by(a, L, rL)) != __float_as_uint(__fdiv_rn(a, L)))
                atomicAdd(bad, 1ull);
        }
}

__global__ void k_x2(const float* p, int pairs, unsigned long long* bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pairs) return;
    const float* q = p + 9 * (size_t)i;  // query, then two points
    const f32x2 d = norm2_rn_x2(pack2(q[0], q[0]), pack2(q[1], q[1]), pack2(q[2], q[2]),
                                pack2(q[3], q[6]), pack2(q[4], q[7]), pack2(q[5], q[8]));
    const float r0 = norm2_rn(q[0], q[1], q[2], q[3], q[4], q[5]);
    const float r1 = norm2_rn(q[0], q[1], q[2], q[6], q[7], q[8]);
    if (__float_as_uint(lo2(d)) != __float_as_uint(r0)) atomicAdd(bad, 1ull);
    if (__float_as_uint(hi2(d)) != __float_as_uint(r1)) atomicAdd(bad, 1ull);
}

int main()
{
    unsigned long long* dbad = nullptr;
    if (cudaMalloc(&dbad, 8) != cudaSuccess) return 2;
    int fails = 0;
    const float Ls[] = {512.0f, 500.0f, 333.3f, 100.1f};
    for (float L : Ls) {
        cudaMemset(dbad, 0, 8);
        k_div<<<152 * 8, 256>>>(0x35800000u, 0x45800000u, L, 1.0f / L, dbad);
        unsigned long long bad = 0;
        const cudaError_t e = cudaMemcpy(&bad, dbad, 8, cudaMemcpyDeviceToHost);
        printf("div L=%g: %s, mismatches %llu\n", L, cudaGetErrorString(e), bad);
        fails += e != cudaSuccess || bad != 0;
    }
    const int pairs = 1 << 21;
    std::vector<float> h(9 * (size_t)pairs);
    uint64_t s = 0x9e3779b97f4a7c15ull;  // xorshift64*
    auto next = [&]() {
        s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
        return (float)((s * 0x2545f4914f6cdd1dull) >> 40) / 16777216.0f;
    };
    for (int i = 0; i < pairs; ++i) {
        float* q = &h[9 * (size_t)i];
        for (int a = 0; a < 3; ++a) q[a] = 1000.0f * next();
        for (int a = 0; a < 6; ++a) q[3 + a] = q[a % 3] + 0.02f * (next() - 0.5f);
    }
    float* dp = nullptr;
    if (cudaMalloc(&dp, 4 * h.size()) != cudaSuccess) return 2;
    cudaMemcpy(dp, h.data(), 4 * h.size(), cudaMemcpyHostToDevice);
    cudaMemset(dbad, 0, 8);
    k_x2<<<(pairs + 255) / 256, 256>>>(dp, pairs, dbad);
    unsigned long long bad = 0;
    const cudaError_t e = cudaMemcpy(&bad, dbad, 8, cudaMemcpyDeviceToHost);
    printf("x2 norm2: %s, mismatches %llu of %d\n", cudaGetErrorString(e), bad, 2 * pairs);
    fails += e != cudaSuccess || bad != 0;
    cudaFree(dp);
    cudaFree(dbad);
    return fails ? 1 : 0;
}
