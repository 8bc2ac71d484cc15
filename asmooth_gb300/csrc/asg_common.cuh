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
constexpr int TIE_MAX = 16;     // exact d2 ties kept per pass of k_knn_ties at the 33rd neighbour

// device error bits (ctx->d_err)
constexpr int ERR_STACK = 1;       // traversal stack overflow
constexpr int ERR_FEW = 2;         // a query found fewer than 33 particles
constexpr int ERR_ZERO_RK = 4;     // 33rd distance is zero (>= 33 coincident particles)
constexpr int ERR_TIES = 8;        // tie selection ran out of passes (not reached for k = 33)
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

// Pairs of floats in one 64-bit register (first element in the low half),
// operated on by the packed f32x2 instructions: one instruction does both IEEE
// single operations, each element rounded to nearest exactly as __fadd_rn /
// __fsub_rn do.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pack2(float lo, float hi)
{
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float lo2(f32x2 v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float hi2(f32x2 v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f32x2 add2_rn(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2_rn(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
// fl(d * d) as one packed fma with a +0 addend.  A packed mul followed by a
// packed add is fused into one fma by the code generator even with explicit
// rounding (measured: a quarter of the sums of two squares differ from the
// scalar __fmul_rn / __fadd_rn result), which the fma form does not allow.  A
// square is never -0, so the +0 addend leaves every rounded product unchanged.
__device__ __forceinline__ f32x2 sq2_rn(f32x2 d)
{
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(r) : "l"(d), "l"(0ull));
    return r;
}

// norm2_rn from the point (ax, ay, az), each coordinate given twice, to two
// points (their x, y and z pairs): the same roundings in the same order
__device__ __forceinline__ f32x2 norm2_rn_x2(f32x2 ax, f32x2 ay, f32x2 az, f32x2 bx, f32x2 by,
                                             f32x2 bz)
{
    const f32x2 dx = sub2_rn(ax, bx), dy = sub2_rn(ay, by), dz = sub2_rn(az, bz);
    return add2_rn(add2_rn(sq2_rn(dx), sq2_rn(dy)), sq2_rn(dz));
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

// The integral of the unit tent max(0, 1 - |t|) over [a, b] (a < b), the cell
// weight of f/ker_integ (coarse_mesh.cpp:10-22), evaluated without
// cancellation.  The reference forms F(b) - F(a) with F(t) = t - t^2/2 (t < 1),
// which cancels when a support ends a sliver inside a cell (0.5 - F(a) for a
// just below 1); here each case uses its factored form, e.g. (1 - a)^2 / 2.
// Every operation is explicitly rounded, so the C restatement in the oracle
// gives the same bits.
__device__ __forceinline__ float tent_pos_rn(float t)  // F(t) for t >= 0
{
    return t >= 1.0f ? 0.5f : __fmul_rn(t, __fsub_rn(1.0f, __fmul_rn(0.5f, t)));
}
__device__ __forceinline__ float tent_integral_rn(float a, float b)
{
    if (a >= 1.0f || b <= -1.0f) return 0.0f;
    if (a >= 0.0f) {  // 0 <= a < 1
        if (b >= 1.0f) {
            const float u = __fsub_rn(1.0f, a);
            return __fmul_rn(__fmul_rn(0.5f, u), u);
        }
        return __fmul_rn(__fsub_rn(b, a), __fsub_rn(1.0f, __fmul_rn(0.5f, __fadd_rn(a, b))));
    }
    if (b <= 0.0f) {  // a < b <= 0
        if (a <= -1.0f) {
            const float u = __fadd_rn(1.0f, b);
            return __fmul_rn(__fmul_rn(0.5f, u), u);
        }
        return __fmul_rn(__fsub_rn(b, a), __fadd_rn(1.0f, __fmul_rn(0.5f, __fadd_rn(a, b))));
    }
    return __fadd_rn(tent_pos_rn(b), tent_pos_rn(-a));  // a < 0 < b
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

// a / L rounded to nearest, given rL = 1/L rounded to nearest: q = RN(a rL) is
// within one ulp of a/L, the residual a - q L is exact as one FMA, and
// RN(q + residual * rL) is the correctly rounded quotient (Markstein's theorem:
// P. W. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1), 1990), for quotients
// and residuals clear of underflow, as the cell edges here are (|a| is a
// position plus or minus a smoothing length, L a box side).  Three operations
// instead of a full division; for a power-of-two L the quotient is exact and
// the residual zero.
__device__ __forceinline__ float div_rn_by(float a, float L, float rL)
{
    const float q = __fmul_rn(a, rL);
    const float r = __fmaf_rn(-q, L, a);
    return __fmaf_rn(r, rL, q);
}

// ---- pruning-only box test --------------------------------------------------
// max of three floats (PTX three-input max, sm_100 and later)
__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Squared distance from a point to an AABB in the cheaper FMA form, for
// pruning only: compare it against prune_bound(t), never against t itself.
// Per axis d = fl(lo - q) (or fl(q - hi)) is at most |fl(p - q)| for every
// point p of the box (rounding is monotone); the FMA sum is at most
// (dx^2 + dy^2 + dz^2)(1 + u)^3 and norm2_rn(q, p) is at least
// (px^2 + py^2 + pz^2)(1 - u)^3 (u = 2^-24), so the result is at most
// norm2_rn(q, p)(1 + 6.1u) for every p in the box.
__device__ __forceinline__ float box_dist2_fast(float qx, float qy, float qz, float lx, float ly,
                                                float lz, float hx, float hy, float hz)
{
    const float dx = max3f(lx - qx, qx - hx, 0.0f);
    const float dy = max3f(ly - qy, qy - hy, 0.0f);
    const float dz = max3f(lz - qz, qz - hz, 0.0f);
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

// the bound that box_dist2_fast is compared against for a threshold t on
// norm2_rn: fl(t (1 + 2^-21)) >= t (1 + 6.9u) > t (1 + 6.1u), so a box holding
// a point with norm2_rn <= t is never pruned (t = +inf stays +inf)
__device__ __forceinline__ float prune_bound(float t) { return __fmul_rn(t, 1.0f + 0x1p-21f); }

// A tree node record (TreeView::rec) holds in words 1-3 either a bucket's own
// box, lo.xyz hi.x | hi.yz, or for a node with more than `leaf` particles the
// boxes of both children as pairs, (lo0.x lo1.x lo0.y lo1.y | lo0.z lo1.z hi0.x
// hi1.x | hi0.y hi1.y hi0.z hi1.z), so that both children are tested with
// packed f32x2 operations.  A leaf child's box is its point, so its distance
// equals norm2_rn to that point.

// a bucket's own box in the fast form
__device__ __forceinline__ float rec_fast0(float4 q, float4 r1, float4 r2)
{
    return box_dist2_fast(q.x, q.y, q.z, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y);
}
// a bucket's own box, rounded as box_dist2_rn
__device__ __forceinline__ float rec_dist0(float4 q, float4 r1, float4 r2)
{
    return box_dist2_rn(q.x, q.y, q.z, make_float4(r1.x, r1.y, r1.z, 0.f),
                        make_float4(r1.w, r2.x, r2.y, 0.f));
}
// both children of a node in the fast form (child 0 low, child 1 high):
// box_dist2_fast's operations on each element; qx = (q.x, q.x) and so on
__device__ __forceinline__ f32x2 node_fast2(f32x2 qx, f32x2 qy, f32x2 qz, float4 r1, float4 r2,
                                            float4 r3)
{
    const f32x2 lx = sub2_rn(pack2(r1.x, r1.y), qx), hx = sub2_rn(qx, pack2(r2.z, r2.w));
    const f32x2 ly = sub2_rn(pack2(r1.z, r1.w), qy), hy = sub2_rn(qy, pack2(r3.x, r3.y));
    const f32x2 lz = sub2_rn(pack2(r2.x, r2.y), qz), hz = sub2_rn(qz, pack2(r3.z, r3.w));
    const f32x2 dx = pack2(max3f(lo2(lx), lo2(hx), 0.0f), max3f(hi2(lx), hi2(hx), 0.0f));
    const f32x2 dy = pack2(max3f(lo2(ly), lo2(hy), 0.0f), max3f(hi2(ly), hi2(hy), 0.0f));
    const f32x2 dz = pack2(max3f(lo2(lz), lo2(hz), 0.0f), max3f(hi2(lz), hi2(hz), 0.0f));
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %1;\n\t"
        "fma.rn.f32x2 %0, %2, %2, %0;\n\t"
        "fma.rn.f32x2 %0, %3, %3, %0;" : "=&l"(r) : "l"(dx), "l"(dy), "l"(dz));
    return r;
}
// child 0 / child 1 of a node, rounded as box_dist2_rn
__device__ __forceinline__ float node_dist0(float4 q, float4 r1, float4 r2, float4 r3)
{
    return box_dist2_rn(q.x, q.y, q.z, make_float4(r1.x, r1.z, r2.x, 0.f),
                        make_float4(r2.z, r3.x, r3.z, 0.f));
}
__device__ __forceinline__ float node_dist1(float4 q, float4 r1, float4 r2, float4 r3)
{
    return box_dist2_rn(q.x, q.y, q.z, make_float4(r1.y, r1.w, r2.y, 0.f),
                        make_float4(r2.w, r3.y, r3.w, 0.f));
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
__host__ __device__ __forceinline__ uint64_t spread3(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Hilbert index of a cell (16 bits per axis), by Skilling's transform
// ("Programming the Hilbert curve", AIP Conf. Proc. 707, 2004): the axes are
// turned into the transposed index by undoing the curve's inversions and
// exchanges level by level, Gray-decoded, then interleaved x-major.  Every
// 3k-bit prefix of the key is one octree cell of level k, as with a Morton
// key, so the radix tree over sorted keys is built the same way; consecutive
// keys are always face-adjacent cells, so 32 consecutive particles are more
// compact than in Morton order.
__host__ __device__ __forceinline__ uint64_t hilbert_key48(uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t X[3] = {x, y, z};
#pragma unroll
    for (uint32_t Q = 1u << 15; Q > 1; Q >>= 1) {
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;  // invert
            } else {        // exchange the low bits of X[0] and X[i]
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    uint32_t t = 0;
#pragma unroll
    for (uint32_t Q = 1u << 15; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    return (spread3(X[0]) << 2) | (spread3(X[1]) << 1) | spread3(X[2]);
}

// ---- warp helpers -------------------------------------------------------------
__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace asg
