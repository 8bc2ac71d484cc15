// asg_knn.cu -- k=33 nearest neighbours, smoothing length and particle density
// (the loop at clumping_tree_main.cpp:418-430 over neighbor_search,
// nbr_search.cpp:61-127, with KNeighbors k=33 from k_neighbors.h:9-51).
//
// Definition implemented (order independent): for query p the neighbour set is
// the 33 particles with the smallest key (d2, input index), d2 evaluated with
// the reference's float expression.  rk = sqrtf(d2 of the 33rd); the 32
// smallest keys (the 33rd excluded, self included) receive the tent weight
// ker(p, q, 1/rk) in dens.
//
// Three warp-bundle kernels over the radix tree (its 64-byte node records); a
// warp serves the 32 consecutive (Hilbert-ordered) particles of one bundle, one
// lane per particle, and visits a node when any lane needs it:
//   k_knn_t33   per-lane sorted top-33 of d2 in registers, candidates queued
//               and merged by comparator networks (asg_knn_net.cuh)
//               -> t33 = 33rd smallest d2 (exact, with multiplicity)
//   k_knn_ties  exact-radius recount: L = #(d2 < t33), the tied indices
//               -> idx33 = input index of the 33rd key, rk = sqrtf(t33)
//   k_dens_scatter the bundle's queries are SOURCES q with their exact radii;
//               in each bucket a lane holds a receiver j and adds ker(q, j)
//               for the queries q whose 32-set holds j, as 64-bit fixed point
//               (per-receiver power-of-two scale, one integer atomic per
//               receiver and bucket): exact integer sums, so deterministic in
//               any order.  It visits the buckets k_knn_t33 recorded.
#include <climits>
#include <type_traits>

#include "asg_common.cuh"
#include "asg_internal.h"
#include "asg_knn_net.cuh"

namespace asg {

constexpr int KNN_WARPS = 4;
// k_knn_t33 runs in blocks of W = 2 or 4 warps (32 warps per SM at 64
// registers either way); in blocks of 2 a warp that finishes early frees its
// slot sooner (23.07 against 23.25 ms on the 256^3 step in Morton order).  The
// batched form's autotuner picks W.
constexpr unsigned FULL = 0xffffffffu;
constexpr int NO_NODE = INT_MIN;  // no node: node ids are >= 0, a leaf i is ~i >= -n

// Merges a lane's queued candidates (KNN_QUEUE values in shared memory, column
// `lane`, +inf where unused) into its ascending top-33 a[] and refills the
// queue with +inf.  tie_out ("a particle outside a[] has d2 == a[32]") stays
// exact: the values dropped by the merge are all >= the 34th smallest t34, so
// one of them ties the new a[32] exactly when t34 == a[32]; an earlier tie
// survives only while a[32] is unchanged.
__device__ __forceinline__ void knn_flush(float (&a)[K_NN], float* qb, float*& qp, bool& tie_out)
{
    float v[KNN_QUEUE];
#pragma unroll
    for (int i = 0; i < KNN_QUEUE; ++i) {
        v[i] = qb[32 * i];
        qb[32 * i] = INFINITY;
    }
    qp = qb;
    knn_sort16(v);
    const float old = a[K_NN - 1];
    const float t34 = knn_merge33(a, v);
    const float top = a[K_NN - 1];
    tie_out = (top == old && tie_out) || t34 == top;
}

// squared distance from the query to a child (point for a leaf child)
__device__ __forceinline__ float child_dist2(const float4* __restrict__ pos, const TreeView& t,
                                             int c, float4 q)
{
    if (c < 0) {
        const float4 p = pos[~c];
        return norm2_rn(q.x, q.y, q.z, p.x, p.y, p.z);
    }
    return box_dist2_rn(q.x, q.y, q.z, t.blo[c], t.bhi[c]);
}

// t33 = the 33rd smallest d2 (with multiplicity), rk = sqrtf(t33), and a tie
// flag: idx33 = -1 when exactly one particle sits at d2 == t33 (then the
// 32-set is {d2 < t33} and needs no index), -2 when ties must be resolved.
// Each lane keeps its 33 smallest d2 sorted in registers; a candidate with
// d2 <= a[32] goes to the lane's queue in shared memory, and when any lane's
// queue holds more than KNN_QUEUE - 2 values after a step of two candidates
// the warp merges every queue with two comparator networks (sort the queue,
// odd-even merge with a[]), about a quarter of the min/max work of inserting
// each candidate as it comes.  Thresholds are the merged a[32], an upper bound
// of the true one while values wait in the queue.  The ids of the buckets
// scanned go to blist for k_dens_scatter.
template <int T33_WARPS>
__global__ void __launch_bounds__(T33_WARPS * 32, 32 / T33_WARPS)
k_knn_t33(const float4* __restrict__ pos, TreeView t, float* __restrict__ t33,
          float* __restrict__ rk, int* __restrict__ idx33, int* __restrict__ blist, int* err)
{
    __shared__ int stk[T33_WARPS][STACK_MAX];
    __shared__ __align__(16) float cand[T33_WARPS][3][32];  // x, y, z of the bucket's particles
    __shared__ float queue[T33_WARPS][KNN_QUEUE][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = t.n;
    const int base = (blockIdx.x * T33_WARPS + warp) * 32;
    if (base >= n) return;
    const int q = min(base + lane, n - 1);
    const float4 xq = pos[q];
    const f32x2 qx = pack2(xq.x, xq.x), qy = pack2(xq.y, xq.y), qz = pack2(xq.z, xq.z);
    float a[K_NN];
#pragma unroll
    for (int k = 0; k < K_NN; ++k) a[k] = INFINITY;
    bool tie_out = false;  // a particle outside a[] has d2 == a[32]
    float* qb = &queue[warp][0][lane];
    float* qp = qb;  // the lane's next free queue slot (qb + 32 x queued values)
#pragma unroll
    for (int i = 0; i < KNN_QUEUE; ++i) qb[32 * i] = INFINITY;
    __shared__ int nlist[T33_WARPS];  // buckets scanned (kept in shared memory: registers are full)
    if (lane == 0) nlist[warp] = 0;

    // the nearer child is visited next without going through the stack; the
    // farther one waits on it
    int* st = stk[warp];
    int sp = 0;
    int next = tree_root(n);
    bool overflow = false;
    for (;;) {
        int node = next;
        next = NO_NODE;
        const bool popped = node == NO_NODE;  // else its box passed the test just now
        if (popped) {
            if (sp == 0) break;
            node = st[--sp];
            __syncwarp();  // every lane has read the slot before it is written again
        }
        int first, last;
        if (node < 0) {
            first = last = ~node;
        } else {
            // the node's record in one round trip: meta and the child boxes (a
            // leaf child's box is its point, so d equals the point's norm2)
            const float4* rp = t.rec + 4 * (size_t)node;
            const float4 r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3];
            const int4 m = make_int4(__float_as_int(r0.x), __float_as_int(r0.y),
                                     __float_as_int(r0.z), __float_as_int(r0.w));
            if (m.w - m.z + 1 > t.leaf) {
                const f32x2 d01 = node_fast2(qx, qy, qz, r1, r2, r3);
                const float d0 = lo2(d01), d1 = hi2(d01);
                const float bound = prune_bound(a[K_NN - 1]);
                // a node whose distance equals a[32] can hold a tie: visit it
                const bool v0 = __any_sync(FULL, d0 <= bound);
                const bool v1 = __any_sync(FULL, d1 <= bound);
                const bool c0_near = __popc(__ballot_sync(FULL, d0 <= d1)) >= 16;
                const int nn = c0_near ? m.x : m.y, ff = c0_near ? m.y : m.x;
                const bool vn = c0_near ? v0 : v1, vf = c0_near ? v1 : v0;
                if (vf) {
                    if (sp + 1 > STACK_MAX) { overflow = true; break; }
                    if (lane == 0) st[sp] = ff;
                    ++sp;
                    __syncwarp();
                }
                if (vn) next = nn;
                continue;
            }
            first = m.z;
            last = m.w;
            // thresholds may have shrunk since the push: re-test a popped bucket
            if (popped && !__any_sync(FULL, rec_fast0(xq, r1, r2) <= prune_bound(a[K_NN - 1])))
                continue;
        }
        if (blist && lane == 0) {
            const int k = nlist[warp];
            if (k < KNN_LIST) blist[(size_t)(base >> 5) * (KNN_LIST + 1) + 1 + k] = node;
            nlist[warp] = k + 1;
        }
        const int cnt = last - first + 1;
        // an odd bucket is padded with a NaN point, whose distance queues nowhere
        if (lane < cnt) {
            const float4 p = pos[first + lane];
            cand[warp][0][lane] = p.x;
            cand[warp][1][lane] = p.y;
            cand[warp][2][lane] = p.z;
        } else if (lane == cnt) {
            cand[warp][0][lane] = __int_as_float(0x7fc00000);
            cand[warp][1][lane] = 0.0f;
            cand[warp][2][lane] = 0.0f;
        }
        __syncwarp();
        // two candidates per step (their distances in packed f32x2 operations),
        // then one check: every queue holds at most KNN_QUEUE - 2 values when a
        // step begins (equal values queue too: the merge tracks ties)
        const f32x2* cx = reinterpret_cast<const f32x2*>(cand[warp][0]);
        const f32x2* cy = reinterpret_cast<const f32x2*>(cand[warp][1]);
        const f32x2* cz = reinterpret_cast<const f32x2*>(cand[warp][2]);
        for (int j = 0; j < cnt; j += 2) {
            const f32x2 d2 = norm2_rn_x2(qx, qy, qz, cx[j >> 1], cy[j >> 1], cz[j >> 1]);
            const float d0 = lo2(d2), d1 = hi2(d2);
            const float top = a[K_NN - 1];
            if (d0 <= top) { *qp = d0; qp += 32; }
            if (d1 <= top) { *qp = d1; qp += 32; }
            if (__any_sync(FULL, qp > qb + 32 * (KNN_QUEUE - 2))) knn_flush(a, qb, qp, tie_out);
        }
        __syncwarp();
    }
    if (__any_sync(FULL, qp > qb)) knn_flush(a, qb, qp, tie_out);
    // every bucket any lane's final radius reaches was scanned, so the list is
    // complete for k_dens_scatter unless it overflowed or the stack did
    if (blist && lane == 0)
        blist[(size_t)(base >> 5) * (KNN_LIST + 1)] =
            (overflow || nlist[warp] > KNN_LIST) ? -1 : nlist[warp];
    if (overflow) {
        if (lane == 0) atomicOr(err, ERR_STACK);
        return;
    }
    if (base + lane < n) {
        const float v = a[K_NN - 1];
        t33[base + lane] = v;
        rk[base + lane] = __fsqrt_rn(v);
        idx33[base + lane] = (tie_out || a[K_NN - 2] == v) ? -2 : -1;
        if (!(v < INFINITY)) atomicOr(err, ERR_FEW);
        else if (!(v > 0.0f)) atomicOr(err, ERR_ZERO_RK);
    }
}

// The 33rd key of flagged queries: with the exact radius T = t33 each lane
// counts L = #(d2 < T) and collects the tied indices (d2 == T); the 33rd key is
// the (33 - L)-th smallest tied index.  A pass keeps the TIE_MAX smallest tied
// indices above a floor (registers, an insertion network); a lane that needs a
// deeper one runs another pass with the floor at its last kept index, so any
// number of ties resolves in at most TIE_PASSES = ceil(33 / TIE_MAX) passes.
constexpr int TIE_PASSES = (K_NN + TIE_MAX - 1) / TIE_MAX;

__global__ void __launch_bounds__(KNN_WARPS * 32)
k_knn_ties(const float4* __restrict__ pos, TreeView t, const float* __restrict__ t33,
           int* __restrict__ idx33, int all, int* err)
{
    __shared__ int stk[KNN_WARPS][STACK_MAX];
    __shared__ float4 cand[KNN_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = t.n;
    const int base = (blockIdx.x * KNN_WARPS + warp) * 32;
    if (base >= n) return;
    const int q = min(base + lane, n - 1);
    // unless every index is wanted, only queries flagged by k_knn_t33 (-2) need it
    const bool want = (base + lane < n) && (all || idx33[q] == -2);
    if (!__any_sync(FULL, want)) return;
    const float4 xq = pos[q];
    const float T = t33[q];
    int nless = 0, neq = 0;
    int need = 0;          // rank of the wanted index among the ties above floor
    int floor_idx = -1;    // this pass keeps tied indices > floor_idx
    bool open = want;      // this lane still looks for its index
    int result = -1;
    int tie[TIE_MAX];
    int* st = stk[warp];

    for (int pass = 0; pass < TIE_PASSES; ++pass) {
        if (!__any_sync(FULL, open)) break;
#pragma unroll
        for (int k = 0; k < TIE_MAX; ++k) tie[k] = INT_MAX;
        if (lane == 0) st[0] = tree_root(n);
        int sp = 1;
        bool overflow = false;
        __syncwarp();
        while (sp > 0) {
            const int node = st[--sp];
            __syncwarp();
            int first, last;
            if (node < 0) {
                first = last = ~node;
            } else {
                const float4* rp = t.rec + 4 * (size_t)node;
                const float4 r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3];
                const int4 m = make_int4(__float_as_int(r0.x), __float_as_int(r0.y),
                                         __float_as_int(r0.z), __float_as_int(r0.w));
                if (m.w - m.z + 1 > t.leaf) {
                    const bool v0 = __any_sync(FULL, open && node_dist0(xq, r1, r2, r3) <= T);
                    const bool v1 = __any_sync(FULL, open && node_dist1(xq, r1, r2, r3) <= T);
                    if (sp + 2 > STACK_MAX) { overflow = true; break; }
                    if (lane == 0) {
                        if (v1) st[sp] = m.y;
                        if (v0) st[sp + (v1 ? 1 : 0)] = m.x;
                    }
                    sp += (v0 ? 1 : 0) + (v1 ? 1 : 0);
                    __syncwarp();
                    continue;
                }
                first = m.z;
                last = m.w;
            }
            const int cnt = last - first + 1;
            if (lane < cnt) cand[warp][lane] = pos[first + lane];
            __syncwarp();
            for (int j = 0; j < cnt; ++j) {
                const float4 c = cand[warp][j];
                const float d2 = norm2_rn(xq.x, xq.y, xq.z, c.x, c.y, c.z);
                if (pass == 0) nless += d2 < T ? 1 : 0;
                const int ci = __float_as_int(c.w);
                const bool eq = open && d2 == T && ci > floor_idx;
                if (__any_sync(FULL, eq)) {
                    if (pass == 0) neq += eq ? 1 : 0;
                    int v = eq ? ci : INT_MAX;
#pragma unroll
                    for (int k = 0; k < TIE_MAX; ++k) {
                        const int lo = min(tie[k], v);
                        v = max(tie[k], v);
                        tie[k] = lo;
                    }
                }
            }
            __syncwarp();
        }
        if (overflow) {
            if (lane == 0) atomicOr(err, ERR_STACK);
            return;
        }
        if (open) {
            if (pass == 0) {
                need = K_NN - nless;  // position of the 33rd key among all the ties
                if (need < 1 || need > neq) {
                    atomicOr(err, ERR_FEW);
                    open = false;
                }
            }
            if (open && need <= TIE_MAX) {
#pragma unroll
                for (int k = 0; k < TIE_MAX; ++k)
                    if (k == need - 1) result = tie[k];
                open = false;
            } else if (open) {
                // the wanted index lies above the TIE_MAX kept ones
                need -= TIE_MAX;
                floor_idx = tie[TIE_MAX - 1];
            }
        }
    }
    if (open) atomicOr(err, ERR_TIES);  // unreachable: need <= 33 <= TIE_PASSES * TIE_MAX
    if (want) idx33[base + lane] = result;
}

// dens is summed as 64-bit fixed point per receiver j: a weight w counts as
// w * 2^(FIX_BITS - e_j), where 2^e_j bounds hinv_j^3.  A query q that has j in
// its 32-set has rk_j <= 2 rk_q (its 33 nearest lie within 2 rk_q of j), so
// w <= hinv_q^3 <= 8 hinv_j^3 and every term stays below 2^(FIX_BITS + 3 + a
// rounding margin).  A lane adds one bucket's terms (at most 32, in query
// order) as a double-float and converts the sum to an integer once; the
// integer atomics make the total independent of the order of the buckets.
constexpr int FIX_BITS = 40;

// e_j with hinv_j^3 < 2^e_j (hinv^3 as the first factor of ker_rn); acc zeroed
__global__ void k_dens_prep(const float* __restrict__ rk, int n, int* __restrict__ dexp,
                            unsigned long long* __restrict__ acc)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float hinv = __fdiv_rn(1.0f, rk[j]);
    const float h3 = __fmul_rn(__fmul_rn(hinv, hinv), hinv);
    const int e = ((__float_as_int(h3) >> 23) & 0xff) - 127 + 1;
    dexp[j] = max(-86, min(86, e));
    acc[j] = 0ull;
}

// The warp serves the 32 queries (sources) q of a bundle with their exact radii
// and visits the buckets k_knn_t33 recorded for the bundle (each re-tested), or
// walks the tree when the list overflowed or is absent.  In a bucket each lane
// holds one candidate receiver j, and the warp loops over only the queries
// whose radius reaches the bucket's box (a ballot; about 9 of 32 on the 256^3
// cube): for each such q every lane tests whether its j is in q's 32-set
// ((d2, index) below q's 33rd key) and adds ker(q, j) as 64-bit fixed point to
// a register; one integer atomic per receiver and bucket adds the sum to
// acc[j].  The sums are exact integers, so the order of the additions and
// atomics does not matter.
__global__ void __launch_bounds__(KNN_WARPS * 32)
k_dens_scatter(const float4* __restrict__ pos, TreeView t, const float* __restrict__ t33,
               const int* __restrict__ idx33, const int* __restrict__ blist,
               const float* __restrict__ rk, const int* __restrict__ dexp,
               unsigned long long* __restrict__ acc, int* __restrict__ err)
{
    __shared__ int stk[KNN_WARPS][STACK_MAX];
    __shared__ float4 qpos[KNN_WARPS][32];  // x, y, z, t33 of the bundle's queries
    __shared__ float4 qaux[KNN_WARPS][32];  // hinv, hinv^3, idx33 (int bits)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = t.n;
    const int base = (blockIdx.x * KNN_WARPS + warp) * 32;
    if (base >= n) return;
    const bool valid = base + lane < n;
    const int q = min(base + lane, n - 1);
    const float4 xq = pos[q];
    const float T = valid ? t33[q] : -1.0f;  // a padding lane takes nothing
    const float hinv = __fdiv_rn(1.0f, rk[q]);
    const float bound = prune_bound(T);
    qpos[warp][lane] = make_float4(xq.x, xq.y, xq.z, T);
    qaux[warp][lane] = make_float4(hinv, __fmul_rn(__fmul_rn(hinv, hinv), hinv),
                                   __int_as_float(idx33[q]), 0.0f);
    __syncwarp();

    // the bucket [first, last] (box from its node record, or a single particle)
    // against the queries of mask M
    // the index rule of the 33rd key only matters in a bundle with a tied query
    const bool any_tie = __any_sync(FULL, valid && idx33[q] >= 0);
    auto scan = [&](int first, int last, unsigned M, auto ties) {
        const int cnt = last - first + 1;
        const bool have = lane < cnt;
        const int j = first + (have ? lane : 0);
        const float4 c = pos[j];
        const float sc = __int_as_float((127 + FIX_BITS - dexp[j]) << 23);  // 2^(FIX_BITS - e_j)
        const int cj = __float_as_int(c.w);
        const f32x2 cxy = pack2(c.x, c.y);
        float sh = 0.0f, sl = 0.0f;  // sum of the scaled weights, double-float
        while (M) {
            const int k = __ffs(M) - 1;
            M &= M - 1;
            const float4 Q = qpos[warp][k];
            const float4 A = qaux[warp][k];
            // norm2 (nbr_search.cpp:20-25) and ker (:27-37) of (q, j), query first;
            // x and y as one packed pair (the same roundings)
            const f32x2 dxy = sub2_rn(pack2(Q.x, Q.y), cxy);
            const float dx = lo2(dxy), dy = hi2(dxy), dz = __fsub_rn(Q.z, c.z);
            const f32x2 sxy = sq2_rn(dxy);
            const float d2 = __fadd_rn(__fadd_rn(lo2(sxy), hi2(sxy)), __fmul_rn(dz, dz));
            bool member = d2 < Q.w;
            if constexpr (decltype(ties)::value) member = member || (d2 == Q.w && cj < __float_as_int(A.z));
            float w = A.y;
            w = __fmul_rn(w, __fsub_rn(1.0f, __fmul_rn(fabsf(dx), A.x)));
            w = __fmul_rn(w, __fsub_rn(1.0f, __fmul_rn(fabsf(dy), A.x)));
            w = __fmul_rn(w, __fsub_rn(1.0f, __fmul_rn(fabsf(dz), A.x)));
            // w * 2^(FIX_BITS - e_j) is exact (a power-of-two scale)
            if (member) two_sum_acc_nonneg(sh, sl, __fmul_rn(w, sc));
        }
        // one conversion per receiver and bucket: hi and lo rounded to integers
        // (lo may be negative; the sum is not)
        const long long sum = __float2ll_rn(sh) + __float2ll_rn(sl);
        if (have && sum) atomicAdd(&acc[j], (unsigned long long)sum);
    };
    // the queries whose radius reaches a bucket node's box
    auto reach = [&](int node) -> unsigned {
        if (node < 0) return __ballot_sync(FULL, valid);
        const float4* rp = t.rec + 4 * (size_t)node;
        return __ballot_sync(FULL, rec_fast0(xq, rp[1], rp[2]) <= bound);
    };
    auto bucket_range = [&](int node, int& first, int& last) {
        if (node < 0) {
            first = last = ~node;
        } else {
            const float4 r0 = t.rec[4 * (size_t)node];
            first = __float_as_int(r0.z);
            last = __float_as_int(r0.w);
        }
    };

    const int* bl = blist ? blist + (size_t)(base >> 5) * (KNN_LIST + 1) : nullptr;
    const int nlist = bl ? bl[0] : -1;
    if (nlist >= 0) {
        // the list in registers: entry i in lane i & 31 of word i >> 5
        int e[(KNN_LIST + 31) / 32];
#pragma unroll
        for (int w = 0; w < (KNN_LIST + 31) / 32; ++w)
            e[w] = 32 * w + lane < nlist ? bl[1 + 32 * w + lane] : 0;
        for (int i = 0; i < nlist; ++i) {
            int v = e[0];
#pragma unroll
            for (int w = 1; w < (KNN_LIST + 31) / 32; ++w)
                if ((i >> 5) == w) v = e[w];
            const int node = __shfl_sync(FULL, v, i & 31);
            const unsigned M = reach(node);
            if (!M) continue;
            int first, last;
            bucket_range(node, first, last);
            if (any_tie) scan(first, last, M, std::true_type{});
            else scan(first, last, M, std::false_type{});
        }
        return;
    }

    int* st = stk[warp];
    if (lane == 0) st[0] = tree_root(n);
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int node = st[--sp];
        __syncwarp();
        if (node >= 0) {
            const int4 m = t.meta[node];
            if (m.w - m.z + 1 > t.leaf) {
                const bool v0 = __any_sync(FULL, child_dist2(pos, t, m.x, xq) <= T);
                const bool v1 = __any_sync(FULL, child_dist2(pos, t, m.y, xq) <= T);
                if (sp + 2 > STACK_MAX) {
                    if (lane == 0) atomicOr(err, ERR_STACK);
                    break;
                }
                if (lane == 0) {
                    if (v1) st[sp] = m.y;
                    if (v0) st[sp + (v1 ? 1 : 0)] = m.x;
                }
                sp += (v0 ? 1 : 0) + (v1 ? 1 : 0);
                __syncwarp();
                continue;
            }
        }
        const unsigned M = reach(node);
        if (!M) continue;
        int first, last;
        bucket_range(node, first, last);
        if (any_tie) scan(first, last, M, std::true_type{});
        else scan(first, last, M, std::false_type{});
    }
}

// dens_j += acc_j * 2^(e_j - FIX_BITS), one rounding to float
__global__ void k_dens_finish(const unsigned long long* __restrict__ acc,
                              const int* __restrict__ dexp, int n, float4* __restrict__ vel)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double scale = __longlong_as_double((long long)(1023 + dexp[j] - FIX_BITS) << 52);
    const float d = __double2float_rn(__dmul_rn(__ull2double_rn(acc[j]), scale));
    float4 v = vel[j];
    v.w = __fadd_rn(v.w, d);  // dens accumulates onto the incoming value, as q->dens += ... does
    vel[j] = v;
}

static int knn_blocks(int n) { return (n + KNN_WARPS * 32 - 1) / (KNN_WARPS * 32); }

void launch_knn_t33(const float4* pos, const TreeView& t, float* t33, float* rk, int* idx33,
                    int* blist, int* err, cudaStream_t s, int warps)
{
    if (t.n <= 0) return;
    if (warps == 4)
        k_knn_t33<4><<<(t.n + 127) / 128, 128, 0, s>>>(pos, t, t33, rk, idx33, blist, err);
    else
        k_knn_t33<2><<<(t.n + 63) / 64, 64, 0, s>>>(pos, t, t33, rk, idx33, blist, err);
    count_launches(1);
}

void launch_knn_ties(const float4* pos, const TreeView& t, const float* t33, int* idx33,
                     int all, int* err, cudaStream_t s)
{
    if (t.n <= 0) return;
    k_knn_ties<<<knn_blocks(t.n), KNN_WARPS * 32, 0, s>>>(pos, t, t33, idx33, all, err);
    count_launches(1);
}

void launch_dens(const float4* pos, const TreeView& t, const float* t33, const int* idx33,
                 const int* blist, const float* rk, int* dexp, unsigned long long* acc,
                 float4* vel, int* err, cudaStream_t s)
{
    if (t.n <= 0) return;
    const int nb = (t.n + 255) / 256;
    k_dens_prep<<<nb, 256, 0, s>>>(rk, t.n, dexp, acc);
    k_dens_scatter<<<knn_blocks(t.n), KNN_WARPS * 32, 0, s>>>(pos, t, t33, idx33, blist, rk, dexp,
                                                             acc, err);
    k_dens_finish<<<nb, 256, 0, s>>>(acc, dexp, t.n, vel);
    count_launches(3);
}

}  // namespace asg
