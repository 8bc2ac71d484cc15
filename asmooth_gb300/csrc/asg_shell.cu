// asg_shell.cu -- the periodic buffer shell of a single-cube run, built on the
// device: what exchange_buffer (exchange_buffer.cpp:13-168) does when one rank
// owns the whole box (every direction a self-exchange), followed by the
// filter of remove_extra_particles (clumping_tree_main.cpp:550-576).
//
// Same particles, same float positions as the reference:
//   bin per axis = (x >= bf*L) + (x > (1-bf)*L)          (exchange_buffer.cpp:6-11)
//   a particle of bin b (b != 13) is copied once per direction d != 13 with
//   d_a == 1 or d_a == b_a on every axis, shifted x -= (d_a - 1)*L   (:120-144)
//   kept when -bf*L < x < L + bf*L on every axis          (clumping_tree_main.cpp:556-566)
// Order of the result: the interior particles as given, then the copies
// grouped by (source bin, direction) in the reference's loop order, each group
// in input order.  (The reference orders a bin by an in-place swap sort, so its
// order within a group differs; no output depends on it except index
// tie-breaks.)
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

__global__ void k_shell_bins(const float4* __restrict__ pos, int n, float lt, float rt,
                             uint32_t* __restrict__ keys, int* __restrict__ vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const int bx = (p.x >= lt) + (p.x > rt);
    const int by = (p.y >= lt) + (p.y > rt);
    const int bz = (p.z >= lt) + (p.z > rt);
    keys[i] = (uint32_t)(bx + 3 * by + 9 * bz);
    vals[i] = i;
}

__global__ void k_shell_bounds(const uint32_t* __restrict__ keys, int n, uint32_t* __restrict__ start,
                               uint32_t* __restrict__ end)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const uint32_t b = keys[m];
    if (m == 0 || keys[m - 1] != b) start[b] = (uint32_t)m;
    if (m == n - 1 || keys[m + 1] != b) end[b] = (uint32_t)m + 1;
}

// interior particles first, unchanged
__global__ void k_shell_interior(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                 const int* __restrict__ igrp, const float* __restrict__ rk, int n,
                                 float4* __restrict__ apos, float4* __restrict__ avel,
                                 int* __restrict__ aigrp, float* __restrict__ ark)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    apos[i] = pos[i];
    avel[i] = vel[i];
    aigrp[i] = igrp[i];
    ark[i] = rk[i];
}

// every copy of the bin-sorted particle m, at its group's offset + rank in the bin
__global__ void k_shell_emit(const float4* __restrict__ pos, const float4* __restrict__ vel,
                             const int* __restrict__ igrp, const float* __restrict__ rk,
                             const uint32_t* __restrict__ keys, const int* __restrict__ order,
                             const uint32_t* __restrict__ start, int n, ShellPlan plan, float L,
                             float4* __restrict__ apos, float4* __restrict__ avel,
                             int* __restrict__ aigrp, float* __restrict__ ark)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const int b = (int)keys[m];
    if (b == 13) return;
    const int i = order[m];
    const uint32_t r = (uint32_t)m - start[b];
    const float4 p = pos[i];
    const float4 v = vel[i];
    const int g = igrp[i];
    const float h = rk[i];
    for (int d = 0; d < 27; ++d) {
        const int base = plan.base[b][d];
        if (base < 0) continue;
        const size_t dst = (size_t)base + r;
        const float sx = __fmul_rn((float)(d % 3 - 1), L);
        const float sy = __fmul_rn((float)((d / 3) % 3 - 1), L);
        const float sz = __fmul_rn((float)(d / 9 - 1), L);
        apos[dst] = make_float4(__fsub_rn(p.x, sx), __fsub_rn(p.y, sy), __fsub_rn(p.z, sz), p.w);
        avel[dst] = v;
        aigrp[dst] = g;
        ark[dst] = h;
    }
}

__global__ void k_shell_keep(const float4* __restrict__ apos, int n, float lo, float hi,
                             uint32_t* __restrict__ flags)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 p = apos[k];
    flags[k] = (lo < p.x && p.x < hi && lo < p.y && p.y < hi && lo < p.z && p.z < hi) ? 1u : 0u;
}

// stable compaction; pos.w becomes the index in the shelled set
__global__ void k_shell_compact(const float4* __restrict__ apos, const float4* __restrict__ avel,
                                const int* __restrict__ aigrp, const float* __restrict__ ark, int n,
                                const uint32_t* __restrict__ scan, float4* __restrict__ pos,
                                float4* __restrict__ vel, int* __restrict__ igrp,
                                float* __restrict__ rk)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || scan[k + 1] == scan[k]) return;
    const uint32_t o = scan[k];
    const float4 p = apos[k];
    pos[o] = make_float4(p.x, p.y, p.z, __int_as_float((int)o));
    vel[o] = avel[k];
    igrp[o] = aigrp[k];
    rk[o] = ark[k];
}

void launch_shell_bins(const float4* pos, int n, float lt, float rt, uint32_t* keys0, int* vals0,
                       uint32_t* keys1, int* vals1, void* sort_tmp, uint32_t* start, uint32_t* end,
                       const uint32_t** keys, const int** order, cudaStream_t s)
{
    cudaMemsetAsync(start, 0, 27 * sizeof(uint32_t), s);
    cudaMemsetAsync(end, 0, 27 * sizeof(uint32_t), s);
    k_shell_bins<<<(n + 255) / 256, 256, 0, s>>>(pos, n, lt, rt, keys0, vals0);
    const int cur = radix_sort32(keys0, vals0, keys1, vals1, n, 5, sort_tmp, s);
    *keys = cur ? keys1 : keys0;
    *order = cur ? vals1 : vals0;
    k_shell_bounds<<<(n + 255) / 256, 256, 0, s>>>(*keys, n, start, end);
    count_launches(2);
}

void launch_shell_emit(const float4* pos, const float4* vel, const int* igrp, const float* rk,
                       const uint32_t* keys, const int* order, const uint32_t* start, int n,
                       const ShellPlan& plan, float L, float4* apos, float4* avel, int* aigrp,
                       float* ark, cudaStream_t s)
{
    k_shell_interior<<<(n + 255) / 256, 256, 0, s>>>(pos, vel, igrp, rk, n, apos, avel, aigrp, ark);
    k_shell_emit<<<(n + 255) / 256, 256, 0, s>>>(pos, vel, igrp, rk, keys, order, start, n, plan, L,
                                                  apos, avel, aigrp, ark);
    count_launches(2);
}

void launch_shell_filter(const float4* apos, const float4* avel, const int* aigrp, const float* ark,
                         int n_all, float lo, float hi, uint32_t* flags, void* scan_tmp,
                         float4* pos, float4* vel, int* igrp, float* rk, cudaStream_t s)
{
    cudaMemsetAsync(flags + n_all, 0, sizeof(uint32_t), s);
    k_shell_keep<<<(n_all + 255) / 256, 256, 0, s>>>(apos, n_all, lo, hi, flags);
    exclusive_scan_u32(flags, (size_t)n_all + 1, scan_tmp, s);
    k_shell_compact<<<(n_all + 255) / 256, 256, 0, s>>>(apos, avel, aigrp, ark, n_all, flags, pos,
                                                         vel, igrp, rk);
    count_launches(2);
}

}  // namespace asg
