// asg_fof.cu -- friends-of-friends groups and SO-halo marking.
//
// FOF (group_fof / link_friends_recursive1, fof.cpp:34-102; remove_small_groups,
// fof.cpp:104-166): two particles are friends when norm2 <= ll*ll in float
// (the reference's predicate, fof.cpp:85-91); groups are the connected
// components.  GPU form: a warp-bundle range search over the radix tree links
// every friend pair (i < j) in a lock-free union-find whose parent pointers
// only ever decrease, so each component's root is its smallest sorted position
// whatever the order of the unions.  Labels 1..ngroup are then assigned in
// order of each group's smallest INPUT index by a scan over input indices
// (membership is bit-exact; the reference numbers groups in kd-tree order).
//
// SO halos (mark_halo_particles, nbr_search.cpp:140-165, driven by the loop at
// clumping_tree_main.cpp:474-485): one warp per halo walks the tree with the
// halo's sphere; lanes test bucket particles with d2 < r*r and set igrp = -1.
#include <climits>

#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

constexpr int FOF_WARPS = 4;
constexpr unsigned FM = 0xffffffffu;
constexpr int UF_LIMIT = 1 << 20;

__device__ __forceinline__ int uf_find(int* P, int x)
{
    for (;;) {
        const int p = __ldcg(P + x);
        if (p == x) return x;
        const int g = __ldcg(P + p);
        if (g == p) return p;
        atomicCAS(P + x, p, g);  // path halving: g is an ancestor of x
        x = g;
    }
}

__device__ __forceinline__ bool uf_union(int* P, int a, int b)
{
    for (int it = 0; it < UF_LIMIT; ++it) {
        int ra = uf_find(P, a), rb = uf_find(P, b);
        if (ra == rb) return true;
        if (ra < rb) { const int t = ra; ra = rb; rb = t; }
        // link the larger root under the smaller one
        if (atomicCAS(P + ra, ra, rb) == ra) return true;
        a = ra;
        b = rb;
    }
    return false;
}

constexpr int NO_NODE = INT_MIN;  // no node: node ids are >= 0, a leaf i is ~i >= -n

__global__ void __launch_bounds__(FOF_WARPS * 32)
k_fof_link(const float4* __restrict__ pos, TreeView t, float ll2, int* P, int* err)
{
    __shared__ int stk[FOF_WARPS][STACK_MAX];
    __shared__ float4 cand[FOF_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = t.n;
    const int base = (blockIdx.x * FOF_WARPS + warp) * 32;
    if (base >= n) return;
    const int q = min(base + lane, n - 1);
    const bool active = base + lane < n;
    const float4 xq = pos[q];
    bool bad = false;

    // child 0 is visited next directly; child 1 waits on the stack
    int* st = stk[warp];
    int sp = 0;
    int next = tree_root(n);
    bool overflow = false;
    for (;;) {
        int node = next;
        next = NO_NODE;
        if (node == NO_NODE) {
            if (sp == 0) break;
            node = st[--sp];
            __syncwarp();  // every lane has read the slot before it is written again
        }
        int first, last;
        if (node < 0) {
            first = last = ~node;
        } else {
            // the node's record: meta and both children's boxes in one round trip
            const float4* rp = t.rec + 4 * (size_t)node;
            const float4 r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3];
            const int4 m = make_int4(__float_as_int(r0.x), __float_as_int(r0.y),
                                     __float_as_int(r0.z), __float_as_int(r0.w));
            if (m.w - m.z + 1 > t.leaf) {
                // child 0 holds [m.z, g] and child 1 [g + 1, m.w]: the radix tree
                // names its children by the split g (node or leaf g, and g + 1)
                const int g = m.x >= 0 ? m.x : ~m.x;
                // only partners with a larger sorted position are linked from q
                const bool n0 = m.x < 0 ? (active && ~m.x > q)
                                        : (active && g > q && node_dist0(xq, r1, r2, r3) <= ll2);
                const bool n1 = m.y < 0 ? (active && ~m.y > q)
                                        : (active && m.w > q && node_dist1(xq, r1, r2, r3) <= ll2);
                const bool v0 = __any_sync(FM, n0);
                const bool v1 = __any_sync(FM, n1);
                if (v1) {
                    if (sp + 1 > STACK_MAX) { overflow = true; break; }
                    if (lane == 0) st[sp] = m.y;
                    ++sp;
                    __syncwarp();
                }
                if (v0) next = m.x;
                continue;
            }
            first = m.z;
            last = m.w;
        }
        const int cnt = last - first + 1;
        if (lane < cnt) cand[warp][lane] = pos[first + lane];
        __syncwarp();
        for (int j = 0; j < cnt; ++j) {
            const int s = first + j;
            const float4 c = cand[warp][j];
            if (active && s > q && norm2_rn(xq.x, xq.y, xq.z, c.x, c.y, c.z) <= ll2)
                bad |= !uf_union(P, q, s);
        }
        __syncwarp();
    }
    if (overflow && lane == 0) atomicOr(err, ERR_STACK);
    if (bad) atomicOr(err, ERR_UF);
}

void launch_fof_link(const float4* pos, const TreeView& t, float ll, int* parent, int* err,
                     cudaStream_t s)
{
    if (t.n <= 0) return;
    const float ll2 = ll * ll;  // host float multiply: fl(ll*ll) as in fof.cpp:86
    k_fof_link<<<(t.n + FOF_WARPS * 32 - 1) / (FOF_WARPS * 32), FOF_WARPS * 32, 0, s>>>(
        pos, t, ll2, parent, err);
    count_launches(1);
}

// P[i] <- root; minin[root] <- min input index; then mark[minin[root]] = 1
__global__ void k_fof_root(const float4* __restrict__ pos, int n, int* P, int* minin)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = uf_find(P, i);
    atomicMin(minin + r, __float_as_int(pos[i].w));
}
__global__ void k_fof_compress(int n, int* P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    P[i] = uf_find(P, i);
}
__global__ void k_fof_mark(int n, const int* P, const int* minin, int* mark)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (P[i] == i) mark[minin[i]] = 1;
}

void launch_fof_finish(const float4* pos, int n, int* parent, int* minin, int* mark,
                       cudaStream_t s)
{
    if (n <= 0) return;
    const int nb = (n + 255) / 256;
    k_fof_root<<<nb, 256, 0, s>>>(pos, n, parent, minin);
    k_fof_compress<<<nb, 256, 0, s>>>(n, parent);
    k_fof_mark<<<nb, 256, 0, s>>>(n, parent, minin, mark);
    count_launches(3);
}

__global__ void k_fof_label(int n, const int* __restrict__ P, const int* __restrict__ minin,
                            const uint32_t* __restrict__ scan, int* __restrict__ igrp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    igrp[i] = (int)scan[minin[P[i]]] + 1;
}

void launch_fof_label(const float4* pos, int n, const int* parent, const int* minin,
                      const uint32_t* scan, int* igrp_sorted, cudaStream_t s)
{
    (void)pos;
    if (n <= 0) return;
    k_fof_label<<<(n + 255) / 256, 256, 0, s>>>(n, parent, minin, scan, igrp_sorted);
    count_launches(1);
}

// remove_small_groups: count members per label, keep labels with >= threshold,
// relabel kept groups 1..nhalo in label order, all others 0
__global__ void k_count_labels(const int* __restrict__ igrp, int n, uint32_t* counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(counts + igrp[i], 1u);
}
void launch_count_labels(const int* igrp, int n, uint32_t* counts, cudaStream_t s)
{
    if (n <= 0) return;
    k_count_labels<<<(n + 255) / 256, 256, 0, s>>>(igrp, n, counts);
    count_launches(1);
}
__global__ void k_keep_mask(uint32_t* counts, int ngrp, int threshold)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ngrp) return;
    counts[g] = (g > 0 && counts[g] >= (uint32_t)threshold) ? 1u : 0u;
}
void launch_keep_mask(uint32_t* counts, int ngrp, int threshold, cudaStream_t s)
{
    k_keep_mask<<<(ngrp + 1 + 255) / 256, 256, 0, s>>>(counts, ngrp, threshold);
    count_launches(1);
}
__global__ void k_relabel(int* igrp, int n, const uint32_t* __restrict__ scan,
                          const uint32_t* __restrict__ keep)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int g = igrp[i];
    igrp[i] = keep[g] ? (int)scan[g] + 1 : 0;
}
void launch_relabel(int* igrp, int n, const uint32_t* scan, const uint32_t* keep, cudaStream_t s)
{
    if (n <= 0) return;
    k_relabel<<<(n + 255) / 256, 256, 0, s>>>(igrp, n, scan, keep);
    count_launches(1);
}

// ---------------------------------------------------------------------------
// SO halos
// ---------------------------------------------------------------------------
constexpr int MH_WARPS = 4;

__global__ void __launch_bounds__(MH_WARPS * 32)
k_mark_halos(const float4* __restrict__ pos, TreeView t, const float* __restrict__ halos, int nh,
             float left, float right, int* __restrict__ igrp, long long* __restrict__ counts,
             double* __restrict__ mass8)
{
    __shared__ int stk[MH_WARPS][STACK_MAX];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int h = blockIdx.x * MH_WARPS + warp;
    if (h >= nh) return;
    const float cx = halos[5 * (size_t)h], cy = halos[5 * (size_t)h + 1],
                cz = halos[5 * (size_t)h + 2], r = halos[5 * (size_t)h + 3],
                mass = halos[5 * (size_t)h + 4];
    const bool inside = left < cx && cx < right && left < cy && cy < right && left < cz && cz < right;
    if (!inside) {
        if (lane == 0) { counts[h] = 0; mass8[h] = 0.0; }
        return;
    }
    const float r2 = __fmul_rn(r, r);
    long long cnt = 0;
    int* st = stk[warp];
    if (lane == 0) st[0] = tree_root(t.n);
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
            // the node's record: a node's children are tested by their boxes before
            // they are pushed, a bucket (or a bucket root) by its own box
            const float4* rp = t.rec + 4 * (size_t)node;
            const float4 r0 = rp[0], r1 = rp[1], r2v = rp[2], r3 = rp[3];
            const int4 m = make_int4(__float_as_int(r0.x), __float_as_int(r0.y),
                                     __float_as_int(r0.z), __float_as_int(r0.w));
            const float4 c4 = make_float4(cx, cy, cz, 0.f);
            if (m.w - m.z + 1 > t.leaf) {
                // a leaf child goes on as a one-particle bucket, tested by its norm2
                const bool v0 = m.x < 0 || node_dist0(c4, r1, r2v, r3) < r2;
                const bool v1 = m.y < 0 || node_dist1(c4, r1, r2v, r3) < r2;
                if (sp + 2 > STACK_MAX) { overflow = true; break; }
                if (lane == 0) {
                    if (v1) st[sp] = m.y;
                    if (v0) st[sp + (v1 ? 1 : 0)] = m.x;
                }
                sp += (v0 ? 1 : 0) + (v1 ? 1 : 0);
                __syncwarp();
                continue;
            }
            if (rec_dist0(c4, r1, r2v) >= r2) continue;
            first = m.z;
            last = m.w;
        }
        const int nb = last - first + 1;
        bool hit = false;
        if (lane < nb) {
            const float4 p = pos[first + lane];
            // norm2(x, particle[i].x) with x the halo centre (nbr_search.cpp:149)
            hit = norm2_rn(cx, cy, cz, p.x, p.y, p.z) < r2;
            if (hit) igrp[first + lane] = -1;
        }
        cnt += __popc(__ballot_sync(FM, hit));
    }
    if (lane == 0) {
        counts[h] = overflow ? -1 : cnt;
        mass8[h] = (double)__fdiv_rn(mass, 8.0f);  // h[i].mass/8.0f (:483)
    }
}

void launch_mark_halos(const float4* pos, const TreeView& t, const float* halos, int nh,
                       float left, float right, int* igrp, long long* counts, double* mass8,
                       cudaStream_t s)
{
    if (nh <= 0 || t.n <= 0) return;
    k_mark_halos<<<(nh + MH_WARPS - 1) / MH_WARPS, MH_WARPS * 32, 0, s>>>(
        pos, t, halos, nh, left, right, igrp, counts, mass8);
    count_launches(1);
}

}  // namespace asg
