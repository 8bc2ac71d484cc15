// asg_common.cuh -- shared device helpers for the GB300 smoothing path.
//
// Exactness rule: every expression whose bits must match the reference
// (distances, kernel weights, cell integrals, cell ranges) is written with the
// explicit round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn), which the compiler never contracts into FMAs, in the same order
// as the reference's C++ expression.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace asg {

constexpr int K_NN = 33;        // KNeighbors::k (k_neighbors.h:47): 32 neighbours + self
constexpr int LEAF_MAX = 32;    // largest bucket: a tree node with <= leaf particles (leaf <= 32) is scanned whole
constexpr int STACK_MAX = 128;  // traversal stack entries per warp
constexpr int TIE_MAX = 16;     // exact d2 ties tracked at the 33rd neighbour

// device error bits (ctx->d_err)
constexpr int ERR_STACK = 1;       // traversal stack overflow
constexpr int ERR_FEW = 2;         // a query found fewer than 33 particles
constexpr int ERR_ZERO_RK = 4;     // 33rd distance is zero (>= 33 coincident particles)
constexpr int ERR_TIES = 8;        // more than TIE_MAX exact ties at the 33rd neighbour
constexpr int ERR_NONFINITE = 16;  // NaN / inf position
constexpr int ERR_UF = 32;         // union-find retry limit hit
constexpr int ERR_RANGE = 64;      // periodic deposit range wider than the mesh
constexpr int ERR_BADCELL = 128;   // mixed-precision cell index outside the grid
constexpr int ERR_CAP = 256;       // more deposit pairs than a pre-sized pair array holds

// ---- exact float helpers (reference expression order) ----------------------

// norm2 (nbr_search.cpp:20-25): ((dx*dx + dy*dy) + dz*dz), no contraction
__device__ __forceinline__ float norm2_rn(float ax, float ay, float az, float bx, float by, float bz)
{
    const float dx = __fsub_rn(ax, bx);
    const float dy = __fsub_rn(ay, by);
    const float dz = __fsub_rn(az, bz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// ker (nbr_search.cpp:27-37): hinv*hinv*hinv*(1-|dx|*hinv)*(1-|dy|*hinv)*(1-|dz|*hinv)
__device__ __forceinline__ float ker_rn(float ax, float ay, float az, float bx, float by, float bz, float hinv)
{
    float w = __fmul_rn(__fmul_rn(hinv, hinv), hinv);
    w = __fmul_rn(w, __fsub_rn(1.0f, __fmul_rn(fabsf(__fsub_rn(ax, bx)), hinv)));
    w = __fmul_rn(w, __fsub_rn(1.0f, __fmul_rn(fabsf(__fsub_rn(ay, by)), hinv)));
    w = __fmul_rn(w, __fsub_rn(1.0f, __fmul_rn(fabsf(__fsub_rn(az, bz)), hinv)));
    return w;
}

// f, ker_integ (coarse_mesh.cpp:10-22): exact cell integral of the unit tent
__device__ __forceinline__ float tent_f_rn(float x)
{
    return x >= 1.0f ? 0.5f : __fsub_rn(x, __fmul_rn(__fmul_rn(0.5f, x), x));
}
__device__ __forceinline__ float ker_integ_rn(float x1, float x2)
{
    const float fac1 = x1 > 0.0f ? 1.0f : -1.0f;
    const float fac2 = x2 > 0.0f ? 1.0f : -1.0f;
    return __fsub_rn(__fmul_rn(fac2, tent_f_rn(__fmul_rn(fac2, x2))),
                     __fmul_rn(fac1, tent_f_rn(__fmul_rn(fac1, x1))));
}

// squared distance from a point to an AABB, rounded so that for every point p
// inside the box norm2_rn(q, p) >= box_dist2_rn(q, box) (rounding is monotone)
__device__ __forceinline__ float box_dist2_rn(float qx, float qy, float qz, float4 lo, float4 hi)
{
    const float dx = fmaxf(fmaxf(__fsub_rn(lo.x, qx), __fsub_rn(qx, hi.x)), 0.0f);
    const float dy = fmaxf(fmaxf(__fsub_rn(lo.y, qy), __fsub_rn(qy, hi.y)), 0.0f);
    const float dz = fmaxf(fmaxf(__fsub_rn(lo.z, qz), __fsub_rn(qz, hi.z)), 0.0f);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// a tree node record's boxes (TreeView::rec words 1-3): child 0 (or a
// bucket's own box) and child 1; a leaf child's box is its point, so the
// distance equals norm2_rn to that point
__device__ __forceinline__ float rec_dist0(float4 q, float4 r1, float4 r2)
{
    return box_dist2_rn(q.x, q.y, q.z, make_float4(r1.x, r1.y, r1.z, 0.f),
                        make_float4(r1.w, r2.x, r2.y, 0.f));
}
__device__ __forceinline__ float rec_dist1(float4 q, float4 r2, float4 r3)
{
    return box_dist2_rn(q.x, q.y, q.z, make_float4(r2.z, r2.w, r3.x, 0.f),
                        make_float4(r3.y, r3.z, r3.w, 0.f));
}

// double-float accumulation (Knuth two-sum): hi + lo carries ~48 bits
// the same (hi, lo) as two_sum_acc for hi >= 0 and x >= 0: Fast2Sum on the
// larger and the smaller operand gives the same rounded sum and the same exact
// error, with a shorter dependency chain
__device__ __forceinline__ void two_sum_acc_nonneg(float& hi, float& lo, float x)
{
    const float a = fmaxf(hi, x), b = fminf(hi, x);
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    hi = s;
    lo = __fadd_rn(lo, e);
}

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

// ---- Morton keys ------------------------------------------------------------
// spread the low 21 bits of v so that bit k lands on bit 3k
__device__ __forceinline__ uint64_t spread3(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// ---- warp helpers -------------------------------------------------------------
__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace asg
