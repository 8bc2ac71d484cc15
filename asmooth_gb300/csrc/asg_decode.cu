// asg_decode.cu -- particle file payloads decoded on the device: the
// conversion loops of read_pm_file_xv (file_reader2.cpp:68-82) and the
// count-prefix expansion of read_pm_file_zip (file_reader2.cpp:187-252).
//
// zip: fine cells of side mesh_scale in (k, j, i) order with x fastest; cell
// c holds zip2[c] particles, or the next int32 of zip3 when zip2[c] == 255.
// A scan of the 255-flags gives each such cell its zip3 entry, a scan of the
// counts gives each cell its first particle, and each particle finds its cell
// by binary search over those offsets.  Per particle and axis, in the
// reference's float order (1-based i):
//   x = mesh_scale*((off + 0.5f)/256.0f + i - 1.0f) - shift,   v = vel / v_r2i
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

__global__ void k_decode_xv(const float* __restrict__ xv, int n, float s0, float s1, float s2,
                            float4* __restrict__ pos, float4* __restrict__ vel,
                            int* __restrict__ igrp, float* __restrict__ rk, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = xv + 6 * (size_t)i;
    const float x = __fsub_rn(r[0], s0), y = __fsub_rn(r[1], s1), z = __fsub_rn(r[2], s2);
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicOr(err, ERR_NONFINITE);
    pos[i] = make_float4(x, y, z, __int_as_float(i));
    vel[i] = make_float4(r[3], r[4], r[5], 0.0f);
    igrp[i] = 0;
    rk[i] = 0.0f;
}

__global__ void k_zip_big(const uint8_t* __restrict__ c8, int ncell, uint32_t* __restrict__ flag)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncell) flag[c] = c8[c] == 255 ? 1u : 0u;
    if (c == ncell) flag[c] = 0u;
}

// counts from the byte counts and, for 255, the cell's zip3 entry (rank = scan of flags)
__global__ void k_zip_counts(const uint8_t* __restrict__ c8, const uint32_t* __restrict__ rank,
                             const int* __restrict__ c32, int n32, int ncell,
                             uint32_t* __restrict__ counts, int* err)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > ncell) return;
    if (c == ncell) {
        counts[c] = 0u;
        return;
    }
    uint32_t k = c8[c];
    if (k == 255u) {
        const uint32_t r = rank[c];
        if (r < (uint32_t)n32 && c32[r] >= 0) {
            k = (uint32_t)c32[r];
        } else {
            atomicOr(err, ERR_BADCELL);
            k = 0u;
        }
    }
    counts[c] = k;
}

__global__ void k_zip_particles(const uint8_t* __restrict__ off, const int16_t* __restrict__ vq,
                                const uint32_t* __restrict__ start, int ncell, int nc, int n,
                                float scale, float v_r2i, float s0, float s1, float s2,
                                float4* __restrict__ pos, float4* __restrict__ vel,
                                int* __restrict__ igrp, float* __restrict__ rk)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    // the cell c with start[c] <= p < start[c + 1] (empty cells have equal starts)
    int lo = 0, hi = ncell - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= (uint32_t)p) lo = mid; else hi = mid - 1;
    }
    const int c = lo;
    const int ci[3] = {c % nc + 1, (c / nc) % nc + 1, c / (nc * nc) + 1};
    const float sh[3] = {s0, s1, s2};
    float x[3], v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float t = __fadd_rn(__fdiv_rn(__fadd_rn((float)off[3 * (size_t)p + d], 0.5f), 256.0f),
                                  (float)ci[d]);
        x[d] = __fsub_rn(__fmul_rn(scale, __fsub_rn(t, 1.0f)), sh[d]);
        v[d] = __fdiv_rn((float)vq[3 * (size_t)p + d], v_r2i);
    }
    pos[p] = make_float4(x[0], x[1], x[2], __int_as_float(p));
    vel[p] = make_float4(v[0], v[1], v[2], 0.0f);
    igrp[p] = 0;
    rk[p] = 0.0f;
}

void launch_decode_xv(const float* xv, int n, const float* shift, float4* pos, float4* vel,
                      int* igrp, float* rk, int* err, cudaStream_t s)
{
    if (n <= 0) return;
    k_decode_xv<<<(n + 255) / 256, 256, 0, s>>>(xv, n, shift[0], shift[1], shift[2], pos, vel, igrp,
                                                 rk, err);
    count_launches(1);
}

size_t zip_scratch_bytes(int ncell)
{
    const size_t C1 = (size_t)ncell + 1;
    return 2 * ((4 * C1 + 255) & ~size_t(255)) + scan_temp_bytes(C1);
}

void launch_zip_counts(const uint8_t* c8, const int* c32, int n32, int ncell, void* scratch,
                       uint32_t** start, int* err, cudaStream_t s)
{
    const size_t C1 = (size_t)ncell + 1, a = (4 * C1 + 255) & ~size_t(255);
    unsigned char* b = static_cast<unsigned char*>(scratch);
    uint32_t* rank = reinterpret_cast<uint32_t*>(b);
    uint32_t* counts = reinterpret_cast<uint32_t*>(b + a);
    void* tmp = b + 2 * a;
    const unsigned grid = (unsigned)((C1 + 255) / 256);
    k_zip_big<<<grid, 256, 0, s>>>(c8, ncell, rank);
    exclusive_scan_u32(rank, C1, tmp, s);
    k_zip_counts<<<grid, 256, 0, s>>>(c8, rank, c32, n32, ncell, counts, err);
    exclusive_scan_u32(counts, C1, tmp, s);  // counts -> first particle of each cell
    count_launches(2);
    *start = counts;
}

void launch_zip_particles(const uint8_t* off, const int16_t* vq, const uint32_t* start, int ncell,
                          int nc, int n, int mesh_scale, float v_r2i, const float* shift,
                          float4* pos, float4* vel, int* igrp, float* rk, cudaStream_t s)
{
    if (n <= 0) return;
    k_zip_particles<<<(n + 255) / 256, 256, 0, s>>>(off, vq, start, ncell, nc, n, (float)mesh_scale,
                                                     v_r2i, shift[0], shift[1], shift[2], pos, vel,
                                                     igrp, rk);
    count_launches(1);
}

}  // namespace asg
