// asg_deposit.cu -- adaptive kernel deposit onto coarse meshes
// (assign_on_mesh, coarse_mesh.cpp:45-127; the periodic assign_on_global_mesh,
// global_mesh.cpp:25-123; the n-only assign_on_density_mesh, :212-269), the
// FP64 mass totals (mesh_total / check_total_mass, coarse_mesh.cpp:35-43,
// clumping_tree_main.cpp:578-600) and the write_mesh_separate normalisation
// (coarse_mesh.cpp:158-171).
//
// Per particle and per cell: the cell range [left, right) per axis is the
// reference's float expression ((x -+ h)/boxsize)*nc, and ker3 = (k0*k1)*k2 as
// in the reference; each 1-D weight k is the tent's integral over the cell,
// evaluated more accurately than the reference's ker_integ(s1, s1 + ds): the
// cell edges' offsets are fma(i, dx, -x)*hinv and the integral uses
// cancellation-free forms (tent_integral_rn).  The reference's float weights
// err by up to 1.1e-5 relative in a mesh cell against FP64 on the 256^3 cube
// (a halo particle's sliver weight in a thin cell); these stay near 1e-6.
//
// Sort by target tile, then gather; deterministic, no atomics on the mesh.
//  (1) k_dep_prep: one record per particle with x, hinv and the normalised
//      edges (x -+ h)/boxsize, which do not depend on nc.
//  (2) k_pair_count / k_pair_emit: every particle emits one (tile, image)
//      pair per 8^3-cell tile its exact cell range touches, at an offset from
//      an exclusive scan (so the emit order is the particle order).
//  (3) a stable radix sort of the pairs by key = tile << 5 | image groups each
//      tile's particles in particle order.
//  (4) k_deposit_items: a persistent kernel whose warps take (tile, segment
//      of seg pairs) work items; a warp accumulates its item in a private
//      shared-memory tile and adds one pair after another, its lanes over the
//      pair's 3-D cell box, so every cell sums its contributions in list
//      order.  k_merge_tiles adds the partial tiles of multi-segment tiles in
//      segment order.
// n, c and halo are double-float (two-sum) sums, so the per-tile FP64 totals
// reproduce the FP64 sum of the float weights.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <utility>
#include <vector>

#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

constexpr int TS = 8;             // tile edge in cells
constexpr int TC = TS * TS * TS;   // cells per tile
constexpr int DEP_THREADS = 256;   // threads of the tile-merge CTA
constexpr int SEG_DEFAULT = 4096;  // pairs per work item unless DepositParams::seg says otherwise
constexpr int PW = 9;              // partial words per cell
constexpr int IMG_BITS = 5;        // periodic images per pair: up to 3 x 3 x 3
// key bits of the image index: none without periodic images (every pair is
// image 0), so the pair sort needs fewer passes
__host__ __device__ inline int img_bits(const DepositParams& P) { return P.periodic ? IMG_BITS : 0; }
constexpr unsigned FULLM = 0xffffffffu;

// ---------------------------------------------------------------------------
// geometry helpers
// ---------------------------------------------------------------------------
struct TileGeo {
    int job, local, nc;
    int O[3], E[3];
};

__device__ __forceinline__ TileGeo tile_geo(const DepositParams& P, int tile)
{
    int jb = 0;
    while (jb + 1 < P.n_jobs && tile >= P.job[jb + 1].tile_begin) ++jb;
    const MeshJob& J = P.job[jb];
    TileGeo g;
    g.job = jb;
    g.local = tile - J.tile_begin;
    g.nc = J.nc;
    const int tx = g.local % J.tiles[0];
    const int ty = (g.local / J.tiles[0]) % J.tiles[1];
    const int tz = g.local / (J.tiles[0] * J.tiles[1]);
    g.O[0] = tx * TS; g.O[1] = ty * TS; g.O[2] = tz * TS;
    for (int a = 0; a < 3; ++a) g.E[a] = min(TS, g.nc - g.O[a]);
    return g;
}

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// cells [left, right) of one axis (unwrapped for the periodic mesh) and the
// mesh images k_lo .. k_lo+nk-1 whose shifted range meets [0, nc)
struct AxisRange {
    int left, right, k_lo, nk;
};

__device__ __forceinline__ AxisRange axis_range(float exlo, float exhi, const MeshJob& J, int nc,
                                                bool periodic)
{
    AxisRange r;
    const float fl = __fmul_rn(exlo, J.ncf);
    const float fr = __fmul_rn(exhi, J.ncf);
    if (!periodic) {  // coarse_mesh.cpp:72-75
        r.left = max(0, __float2int_rz(fl));
        r.right = min(nc, 1 + __float2int_rz(fr));
        r.k_lo = 0;
        r.nk = r.left < r.right ? 1 : 0;
    } else {  // global_mesh.cpp:66-69; cells wrap modulo nc (:85-87)
        r.left = (int)floorf(fl);
        r.right = 1 + (int)ceilf(fr);
        r.k_lo = floor_div(r.left, nc);
        r.nk = floor_div(r.right - 1, nc) - r.k_lo + 1;
    }
    return r;
}

// ---------------------------------------------------------------------------
// (1) per-particle records
// ---------------------------------------------------------------------------
constexpr int FLAG_HALO = 1;  // sign*igrp > 0: deposit into the halo channel
constexpr int FLAG_SKIP = 2;  // periodic particle outside [0, L) or a halo in an n-only mesh

// One 32-byte record per particle: (x', y', z', h') and (dens, vx, vy, vz),
// with x' the deposit position (plus the rank offset when periodic) and h' = h,
// -h when the particle deposits into the halo channel, 0 when it deposits
// nothing.  The cell-range edges (x' -+ h)/L and 1/h are recomputed from it
// where they are needed (load_dep_rec), with the same rounded operations.
__global__ void k_dep_prep(const float4* __restrict__ pos, const float4* __restrict__ vel,
                           const int* __restrict__ igrp, const float* __restrict__ rk, int n,
                           DepositParams P, float4* __restrict__ rec, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const float4 v = vel[i];
    const float h = rk[i];
    if (!(h > 0.0f && h < INFINITY)) atomicOr(err, ERR_ZERO_RK);
    const float L = P.boxsize;
    const bool halo = (P.sign * igrp[i]) > 0;
    bool skip = P.density_only && halo;
    float x = p.x, y = p.y, z = p.z;
    if (P.periodic) {  // global_mesh.cpp:52-61: skip outside the cube, then add the offset
        if (x < 0.0f || x >= L || y < 0.0f || y >= L || z < 0.0f || z >= L) skip = true;
        x = __fadd_rn(x, P.offset[0]);
        y = __fadd_rn(y, P.offset[1]);
        z = __fadd_rn(z, P.offset[2]);
    }
    if (!(h > 0.0f && h < INFINITY)) skip = true;
    rec[2 * (size_t)i] = make_float4(x, y, z, skip ? 0.0f : (halo ? -h : h));
    rec[2 * (size_t)i + 1] = make_float4(v.w, v.x, v.y, v.z);
}

// particle i's record as the deposit kernels use it: A = (x', 1/h), B = ((x'-h)/L,
// dens), Cc = ((x'+h)/L, vx), D = (vy, vz, flags)
__device__ __forceinline__ void load_dep_rec(const float4* __restrict__ rec, int i, float L,
                                             float rL, float4& A, float4& B, float4& Cc, float4& D)
{
    const float4 a = rec[2 * (size_t)i], b = rec[2 * (size_t)i + 1];
    const float h = fabsf(a.w);
    const int flags = (a.w < 0.0f ? FLAG_HALO : 0) | (h > 0.0f ? 0 : FLAG_SKIP);
    A = make_float4(a.x, a.y, a.z, __frcp_rn(h));  // 1/h correctly rounded
    B = make_float4(div_rn_by(__fsub_rn(a.x, h), L, rL), div_rn_by(__fsub_rn(a.y, h), L, rL),
                    div_rn_by(__fsub_rn(a.z, h), L, rL), b.x);
    Cc = make_float4(div_rn_by(__fadd_rn(a.x, h), L, rL), div_rn_by(__fadd_rn(a.y, h), L, rL),
                     div_rn_by(__fadd_rn(a.z, h), L, rL), b.y);
    D = make_float4(b.z, b.w, __int_as_float(flags), 0.0f);
}

// ---------------------------------------------------------------------------
// (2) (tile, image) pairs
// ---------------------------------------------------------------------------
// tiles of one axis touched by image k: [t0, t1] (empty when t0 > t1)
__device__ __forceinline__ void image_tiles(const AxisRange& r, int k, int nc, int& t0, int& t1)
{
    const int c0 = max(r.left - k * nc, 0), c1 = min(r.right - k * nc, nc);
    t0 = c0 / TS;
    t1 = c1 > c0 ? (c1 - 1) / TS : t0 - 1;
}

// EMIT writes pair o only when o < cap (the pair arrays' capacity); a pair
// beyond it sets ERR_CAP instead
template <bool EMIT>
__global__ void k_pairs(const float4* __restrict__ rec, int n, DepositParams P,
                        uint32_t* __restrict__ counts, const uint32_t* __restrict__ offs,
                        uint32_t* __restrict__ keys, int* __restrict__ vals, uint32_t cap, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a, b, c, d;
    load_dep_rec(rec, i, P.boxsize, P.rbox, a, b, c, d);
    const int flags = __float_as_int(d.z);
    uint32_t cnt = 0;
    uint32_t o = EMIT ? offs[i] : 0u;
    const bool periodic = P.periodic != 0;
    if (!(flags & FLAG_SKIP)) {
        for (int jb = 0; jb < P.n_jobs; ++jb) {
            const MeshJob& J = P.job[jb];
            const int nc = J.nc;
            const AxisRange ax = axis_range(b.x, c.x, J, nc, periodic);
            const AxisRange ay = axis_range(b.y, c.y, J, nc, periodic);
            const AxisRange az = axis_range(b.z, c.z, J, nc, periodic);
            if (ax.nk <= 0 || ay.nk <= 0 || az.nk <= 0) continue;
            if (ax.nk > 3 || ay.nk > 3 || az.nk > 3) {  // support wider than two mesh periods
                atomicOr(err, ERR_RANGE);
                continue;
            }
            for (int dz = 0; dz < az.nk; ++dz) {
                int z0, z1;
                image_tiles(az, az.k_lo + dz, nc, z0, z1);
                for (int dy = 0; dy < ay.nk; ++dy) {
                    int y0, y1;
                    image_tiles(ay, ay.k_lo + dy, nc, y0, y1);
                    for (int dx = 0; dx < ax.nk; ++dx) {
                        int x0, x1;
                        image_tiles(ax, ax.k_lo + dx, nc, x0, x1);
                        if (x0 > x1 || y0 > y1 || z0 > z1) continue;
                        const uint32_t combo = (uint32_t)(dz * 9 + dy * 3 + dx);
                        if constexpr (!EMIT) {
                            cnt += (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1));
                        } else {
                            for (int tz = z0; tz <= z1; ++tz)
                                for (int ty = y0; ty <= y1; ++ty)
                                    for (int tx = x0; tx <= x1; ++tx) {
                                        const uint32_t tile = (uint32_t)J.tile_begin +
                                            (uint32_t)((tz * J.tiles[1] + ty) * J.tiles[0] + tx);
                                        if (o < cap) {
                                            keys[o] = (tile << img_bits(P)) | combo;
                                            vals[o] = i;
                                        } else {
                                            atomicOr(err, ERR_CAP);
                                        }
                                        ++o;
                                    }
                        }
                    }
                }
            }
        }
    }
    if (!EMIT) counts[i] = cnt;
}

// pairs [*npairs, cap) of a pre-sized pair array: key of tile T (past the last
// real tile), so they sort last and k_tile_bounds skips them
__global__ void k_pad_pairs(uint32_t* __restrict__ keys, int* __restrict__ vals,
                            const uint32_t* __restrict__ npairs, uint32_t cap, uint32_t pad_key)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cap || j < *npairs) return;
    keys[j] = pad_key;
    vals[j] = 0;
}

// first pair and pair count of every tile (sorted keys; empty tiles stay 0;
// tiles >= total_tiles are padding)
__global__ void k_tile_bounds(const uint32_t* __restrict__ keys, int np, int total_tiles, int ib,
                              uint32_t* __restrict__ tstart, uint32_t* __restrict__ tcount)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= np) return;
    const uint32_t t = keys[j] >> ib;
    if (t >= (uint32_t)total_tiles) return;
    if (j == 0 || (keys[j - 1] >> ib) != t) tstart[t] = (uint32_t)j;
    if (j == np - 1 || (keys[j + 1] >> ib) != t) tcount[t] = (uint32_t)j + 1;  // end for now
}

// tcount: end -> count; nitems: seg-pair work items per tile (at least one),
// stored at the tile's slot of the processing order (DepositParams::pos)
__global__ void k_tile_items(const uint32_t* __restrict__ tstart, uint32_t* __restrict__ tcount,
                             int total_tiles, int seg, const uint32_t* __restrict__ pos,
                             uint32_t* __restrict__ nitems)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total_tiles) {
        const uint32_t c = tcount[i] ? tcount[i] - tstart[i] : 0u;
        tcount[i] = c;
        nitems[pos ? pos[i] : (uint32_t)i] = max(1u, (c + (uint32_t)seg - 1) / (uint32_t)seg);
    }
    if (i == total_tiles) nitems[i] = 0u;
}

// ---------------------------------------------------------------------------
// (4) persistent deposit of (tile, segment) work items
// ---------------------------------------------------------------------------
// One warp owns one work item and accumulates its tile in a private
// shared-memory copy; it adds the item's pairs one after another, its lanes
// spread over the pair's whole 3-D cell box.  Per cell the additions happen in
// pair order, so the sums are deterministic.
constexpr int DEP_WARPS = 2;                // warps per CTA (independent)
constexpr int WROW = 3 * TS + 1;            // staged 1-D weights per lane: [axis * TS + cell]

struct WarpTile {
    float4 a[TC];           // n_hi, n_lo, c_hi, c_lo
    float4 b[TC];           // vx, vy, vz, halo_hi
    float hl[TC];           // halo_lo
    float w[32][WROW];      // 1-D cell weights of the chunk's 32 pairs (odd row stride)
};

// cell slot in a WarpTile: rows of 8 cells rotated by (6y + 4z) mod 8, which
// spreads the 128-bit accesses of a small 3-D box over distinct bank groups
__device__ __forceinline__ int tile_slot(int x, int y, int z)
{
    return (z << 6) | (y << 3) | ((x + 6 * y + 4 * z) & (TS - 1));
}

// floor(c / d) = (c * m_d) >> 15 with m_d = ceil(2^15 / d), exactly for
// 0 <= c < 512 and 1 <= d <= 64 (checked for every c and d): a pair's box has
// at most 8^3 cells and nx * ny <= 64.  Integer multiply and shift, no
// conversions on the per-cell path.
#define ASG_M15(d) ((32768 + (d) - 1) / (d))
#define ASG_M8(b) ASG_M15(b + 1), ASG_M15(b + 2), ASG_M15(b + 3), ASG_M15(b + 4), \
    ASG_M15(b + 5), ASG_M15(b + 6), ASG_M15(b + 7), ASG_M15(b + 8)
__constant__ int c_m15[TS * TS + 1] = {0, ASG_M8(0), ASG_M8(8), ASG_M8(16), ASG_M8(24),
                                       ASG_M8(32), ASG_M8(40), ASG_M8(48), ASG_M8(56)};
#undef ASG_M8
#undef ASG_M15

__device__ __forceinline__ int small_div(int c, int m) { return (c * m) >> 15; }

// one particle's weight w3 into one cell: n and c as double-float, v as float
__device__ __forceinline__ void add_cell(WarpTile& S, int slot, float w3, float dens, float vx,
                                         float vy, float vz)
{
    float4 Aa = S.a[slot];
    float4 Bb = S.b[slot];
    two_sum_acc_nonneg(Aa.x, Aa.y, w3);
    const float pr = __fmul_rn(w3, dens);
    const float pe = fmaf(w3, dens, -pr);  // the exact rounding error of the product
    two_sum_acc_nonneg(Aa.z, Aa.w, pr);
    Aa.w = __fadd_rn(Aa.w, pe);
    Bb.x = fmaf(w3, vx, Bb.x);
    Bb.y = fmaf(w3, vy, Bb.y);
    Bb.z = fmaf(w3, vz, Bb.z);
    S.a[slot] = Aa;
    S.b[slot] = Bb;
}

// a halo particle's weight into the halo channel (double-float)
__device__ __forceinline__ void add_halo(WarpTile& S, int slot, float w3)
{
    float hh = S.b[slot].w, hl = S.hl[slot];
    two_sum_acc_nonneg(hh, hl, w3);
    S.b[slot].w = hh;
    S.hl[slot] = hl;
}

__device__ __forceinline__ int upper_index(const uint32_t* __restrict__ a, int n, uint32_t v)
{
    // largest i in [0, n) with a[i] <= v (a non-decreasing, a[0] = 0)
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void write_tile(const WarpTile& S, const DepositParams& P, const TileGeo& g,
                                           double& sn, double& sh, int lane)
{
    const MeshJob& J = P.job[g.job];
    const int nc = g.nc;
    const size_t nmesh = (size_t)nc * nc * nc;
    for (int e = lane; e < TC; e += 32) {
        const int lz = e >> 6, ly = (e >> 3) & (TS - 1), lx = e & (TS - 1);
        if (lx >= g.E[0] || ly >= g.E[1] || lz >= g.E[2]) continue;
        const int slot = tile_slot(lx, ly, lz);
        const float4 A = S.a[slot];
        const float4 B = S.b[slot];
        const float hl = S.hl[slot];
        const size_t idx = ((size_t)(g.O[2] + lz) * nc + (g.O[1] + ly)) * nc + (g.O[0] + lx);
        sn += (double)A.x + (double)A.y;
        sh += (double)B.w + (double)hl;
        J.mesh[idx] = __fadd_rn(A.x, A.y);
        if (!P.density_only) {
            J.mesh[nmesh + idx] = __fadd_rn(B.w, hl);
            J.mesh[2 * nmesh + idx] = __fadd_rn(A.z, A.w);
            J.mesh[3 * nmesh + 3 * idx] = B.x;
            J.mesh[3 * nmesh + 3 * idx + 1] = B.y;
            J.mesh[3 * nmesh + 3 * idx + 2] = B.z;
        }
    }
}

__device__ __forceinline__ void block_totals(double sn, double sh, double (*red)[DEP_THREADS / 32],
                                             const MeshJob& J, int local, int tid)
{
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sn += __shfl_down_sync(FULLM, sn, o);
        sh += __shfl_down_sync(FULLM, sh, o);
    }
    if (lane == 0) {
        red[0][warp] = sn;
        red[1][warp] = sh;
    }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < DEP_THREADS / 32; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        J.partial[2 * local] = a;
        J.partial[2 * local + 1] = b;
    }
}

__global__ void __launch_bounds__(32 * DEP_WARPS)
k_deposit_items(const float4* __restrict__ rec, DepositParams P, int total_tiles,
                const uint32_t* __restrict__ item_off, const uint32_t* __restrict__ tstart,
                const uint32_t* __restrict__ tcount, const uint32_t* __restrict__ pkeys,
                const int* __restrict__ pvals, float* __restrict__ partial,
                int* __restrict__ next_item)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    WarpTile& S = reinterpret_cast<WarpTile*>(smem_raw)[threadIdx.x >> 5];
    const bool periodic = P.periodic != 0;
    const uint32_t total_items = item_off[total_tiles];

    for (;;) {
        int item = 0, tile = -1;
        if (lane == 0) {
            item = atomicAdd(next_item, 1);
            if ((uint32_t)item < total_items) tile = upper_index(item_off, total_tiles + 1, (uint32_t)item);
        }
        item = __shfl_sync(FULLM, item, 0);
        const int slot = __shfl_sync(FULLM, tile, 0);  // items are numbered in slot order
        if ((uint32_t)item >= total_items) break;
        tile = P.order ? (int)P.order[slot] : slot;
        const TileGeo g = tile_geo(P, tile);
        const MeshJob& J = P.job[g.job];
        const int nc = g.nc;
        const int seg = item - (int)item_off[slot];
        const int nseg = (int)(item_off[slot + 1] - item_off[slot]);
        const int j0 = (int)tstart[tile] + seg * P.seg;
        const int j1 = (int)tstart[tile] + min((int)tcount[tile], (seg + 1) * P.seg);

        for (int e = lane; e < TC; e += 32) {
            S.a[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            S.b[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            S.hl[e] = 0.f;
        }
        __syncwarp();

        for (int c0 = j0; c0 < j1; c0 += 32) {
            // ---- setup: one pair per lane: exact ranges of its image, 1-D weights ----
            // rect packs tile-relative [x0,x1) [y0,y1) [z0,z1) in 4-bit fields and
            // the halo flag in bit 24; 0 means no cells
            uint32_t rect = 0;
            float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
            {
                const int j = c0 + lane;
                if (j < j1) {
                    const int i = pvals[j];
                    const int combo = P.periodic ? (int)(pkeys[j] & ((1u << IMG_BITS) - 1u)) : 0;
                    const int dk[3] = {combo % 3, (combo / 3) % 3, combo / 9};
                    float4 A, B, Cc, D;
                    load_dep_rec(rec, i, P.boxsize, P.rbox, A, B, Cc, D);
                    const float xs[3] = {A.x, A.y, A.z};
                    const float lo[3] = {B.x, B.y, B.z};
                    const float hi[3] = {Cc.x, Cc.y, Cc.z};
                    const float hinv = A.w;
                    float* wl = S.w[lane];
                    uint32_t r = 0;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const AxisRange ar = axis_range(lo[a], hi[a], J, nc, periodic);
                        const int k = ar.k_lo + dk[a];
                        const int sh = k * nc + g.O[a];
                        const int r0 = max(ar.left - sh, 0), r1 = min(ar.right - sh, g.E[a]);
                        r |= (uint32_t)((r0 & 15) | ((max(r1, r0) & 15) << 4)) << (8 * a);
                        // cell t covers [fi*dx, (fi+1)*dx] for the unwrapped cell index
                        // fi = t + sh (exact float steps, |index| < 2^24); each edge's
                        // offset from the particle in units of h is fma(fi, dx, -x) * hinv
                        // (one rounding before the scaling; the reference's s1 and
                        // s1 + ds, coarse_mesh.cpp:80-90, round i*dx first)
                        float fi = (float)(r0 + sh);
                        float e0 = __fmul_rn(__fmaf_rn(fi, J.dx, -xs[a]), hinv);
                        for (int t = r0; t < r1; ++t) {
                            fi = __fadd_rn(fi, 1.0f);
                            const float e1 = __fmul_rn(__fmaf_rn(fi, J.dx, -xs[a]), hinv);
                            wl[a * TS + t] = tent_integral_rn(e0, e1);
                            e0 = e1;
                        }
                    }
                    rect = r | ((uint32_t)(__float_as_int(D.z) & FLAG_HALO) << 24);
                    val = make_float4(B.w, Cc.w, D.x, D.y);
                }
            }
            __syncwarp();
            // ---- the warp adds the chunk's pairs in order, lanes over each pair's cells ----
            const int cnt = min(32, j1 - c0);
            for (int p = 0; p < cnt; ++p) {
                const uint32_t rp = __shfl_sync(FULLM, rect, p);
                const int x0 = rp & 15, nx = ((rp >> 4) & 15) - x0;
                const int y0 = (rp >> 8) & 15, ny = ((rp >> 12) & 15) - y0;
                const int z0 = (rp >> 16) & 15, nz = ((rp >> 20) & 15) - z0;
                if (nx <= 0 || ny <= 0 || nz <= 0) continue;
                const float dens = __shfl_sync(FULLM, val.x, p);
                const float vx = __shfl_sync(FULLM, val.y, p);
                const float vy = __shfl_sync(FULLM, val.z, p);
                const float vz = __shfl_sync(FULLM, val.w, p);
                const int nxy = nx * ny, ncell = nxy * nz;
                const int rx = c_m15[nx], rxy = c_m15[nxy];
                const float* wp = S.w[p];
                const bool hal = (rp >> 24) != 0;
                if (!hal) {
                    for (int c = lane; c < ncell; c += 32) {
                        const int iz = small_div(c, rxy);
                        const int rem = c - iz * nxy;
                        const int iy = small_div(rem, rx);
                        const int gx = x0 + rem - iy * nx, gy = y0 + iy, gz = z0 + iz;
                        const float w3 = __fmul_rn(__fmul_rn(wp[gx], wp[TS + gy]), wp[2 * TS + gz]);
                        add_cell(S, tile_slot(gx, gy, gz), w3, dens, vx, vy, vz);
                    }
                } else {
                    for (int c = lane; c < ncell; c += 32) {
                        const int iz = small_div(c, rxy);
                        const int rem = c - iz * nxy;
                        const int iy = small_div(rem, rx);
                        const int gx = x0 + rem - iy * nx, gy = y0 + iy, gz = z0 + iz;
                        const float w3 = __fmul_rn(__fmul_rn(wp[gx], wp[TS + gy]), wp[2 * TS + gz]);
                        add_halo(S, tile_slot(gx, gy, gz), w3);
                    }
                }
                __syncwarp();  // the next pair may add to the same cells from other lanes
            }
            __syncwarp();  // the next chunk's setup overwrites S.w
        }

        // ---- write: final tile when alone, partial tile otherwise ----
        if (nseg > 1) {
            float* pt = partial + (size_t)item * TC * PW;
            for (int e = lane; e < TC; e += 32) {
                const int slot = tile_slot(e & (TS - 1), (e >> 3) & (TS - 1), e >> 6);
                const float4 A = S.a[slot];
                const float4 B = S.b[slot];
                pt[e] = A.x; pt[TC + e] = A.y; pt[2 * TC + e] = A.z; pt[3 * TC + e] = A.w;
                pt[4 * TC + e] = B.x; pt[5 * TC + e] = B.y; pt[6 * TC + e] = B.z;
                pt[7 * TC + e] = B.w; pt[8 * TC + e] = S.hl[slot];
            }
        } else {
            double sn = 0.0, sh = 0.0;
            write_tile(S, P, g, sn, sh, lane);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sn += __shfl_down_sync(FULLM, sn, o);
                sh += __shfl_down_sync(FULLM, sh, o);
            }
            if (lane == 0) {
                J.partial[2 * g.local] = sn;
                J.partial[2 * g.local + 1] = sh;
            }
        }
        __syncwarp();  // the next item clears the tile
    }
}

// ---------------------------------------------------------------------------
// (4') the same work items on the tensor cores
// ---------------------------------------------------------------------------
// A pair's contribution to its tile is separable: weight wx[x] wy[y] wz[z]
// times the particle's value in each channel (n: 1, halo: 1, c: dens, v), so a
// tile is a sum of outer products, C[(x, y)][(channel, z)] = sum over pairs of
// A[(x, y)][p] B[p][(channel, z)] with A = wx wy (64 rows) and B = wz * value
// (8 columns per channel): a GEMM with K = the item's pairs.  One warp runs it
// with mma.sync m16n8k8 (TF32 in, FP32 accumulate), 8 pairs per K step, 4 x
// NCH fragments of 16 x 8 held in registers.  TF32 keeps 11 significant bits,
// so every operand is split into hi + lo TF32 parts and each K step issues
// lo*hi, hi*lo and hi*hi (the lo*lo term is below 2^-22 relative), which
// gives each product to about 2^-21.  Every 64 pairs the fragments are added
// into per-lane double-float sums in shared memory and cleared, so the FP32
// accumulation never carries more than 24 roundings.  Lane (g, t) owns the
// cells x = g, z = 2t + {0, 1} and every y of the tile, both in the fragments
// and in its sums, so the sums need no synchronisation.
// The FP64 mass totals do not come from the cells: each pair adds
// (sum wx)(sum wy)(sum wz), formed in double-float arithmetic, to its lane's
// double-float total.  A K step skips the row blocks (two y rows each) and the
// channels that none of its 8 pairs touches: their products are exact zeros.
constexpr int MMA_WARPS = 2;
constexpr int MMA_FLUSH = 64;  // pairs between flushes of the fragments
constexpr uint32_t INFO_MAIN = 1u << 8;  // a pair deposits into n, c and v
constexpr uint32_t INFO_HALO = 1u << 9;  // a pair deposits into halo

template <int NCH>
struct MmaWarp {
    float acc[NCH == 1 ? 2 : 9][16][32];  // [word][2 y + dz][lane]: n hi/lo, c hi/lo, halo hi/lo, v xyz
    float w[32][WROW];                    // per pair of the chunk: wx[0..7] | wy[0..7] | wz[0..7]
    float v[32][NCH == 1 ? 1 : 8];        // per pair: n, halo, c, vx, vy, vz values
};

__device__ __forceinline__ uint32_t tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
// x = hi + lo: hi = x rounded to TF32 (11 significant bits), lo = x - hi
// (exact in FP32) passed with its FP32 bits: the tensor core reads the TF32
// part of an operand register, so lo enters truncated to 11 significant bits,
// an error below 2^-11 |lo| <= 2^-23 |x|
__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo)
{
    hi = tf32_rna(x);
    lo = __float_as_uint(__fsub_rn(x, __uint_as_float(hi)));
}
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// double-float (hi, lo) helpers in FP32 arithmetic: exact product of a
// double-float and a float (two_prod by FMA), and accumulation
__device__ __forceinline__ void df_mul(float& hi, float& lo, float b)
{
    const float p = __fmul_rn(hi, b);
    const float e = fmaf(hi, b, -p);
    hi = p;
    lo = fmaf(lo, b, e);
}
__device__ __forceinline__ void df_mul_df(float& hi, float& lo, float bh, float bl)
{
    const float p = __fmul_rn(hi, bh);
    const float e = fmaf(hi, bh, -p);
    const float l = fmaf(hi, bl, fmaf(lo, bh, e));
    const float s = __fadd_rn(p, l);
    lo = __fsub_rn(l, __fsub_rn(s, p));
    hi = s;
}

template <int NCH>
__global__ void __launch_bounds__(32 * MMA_WARPS)
k_deposit_mma(const float4* __restrict__ rec, DepositParams P, int total_tiles,
              const uint32_t* __restrict__ item_off, const uint32_t* __restrict__ tstart,
              const uint32_t* __restrict__ tcount, const uint32_t* __restrict__ pkeys,
              const int* __restrict__ pvals, float* __restrict__ partial,
              double* __restrict__ item_tot, int* __restrict__ next_item)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NW = NCH == 1 ? 2 : 9;
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    MmaWarp<NCH>& S = reinterpret_cast<MmaWarp<NCH>*>(smem_raw)[threadIdx.x >> 5];
    const bool periodic = P.periodic != 0;
    const uint32_t total_items = item_off[total_tiles];

    for (;;) {
        int item = 0, tile = -1;
        if (lane == 0) {
            item = atomicAdd(next_item, 1);
            if ((uint32_t)item < total_items) tile = upper_index(item_off, total_tiles + 1, (uint32_t)item);
        }
        item = __shfl_sync(FULLM, item, 0);
        const int slot = __shfl_sync(FULLM, tile, 0);  // items are numbered in slot order
        if ((uint32_t)item >= total_items) break;
        tile = P.order ? (int)P.order[slot] : slot;
        const TileGeo geo = tile_geo(P, tile);
        const MeshJob& J = P.job[geo.job];
        const int nc = geo.nc;
        const int seg = item - (int)item_off[slot];
        const int nseg = (int)(item_off[slot + 1] - item_off[slot]);
        const int j0 = (int)tstart[tile] + seg * P.seg;
        const int j1 = (int)tstart[tile] + min((int)tcount[tile], (seg + 1) * P.seg);

#pragma unroll
        for (int k = 0; k < NW; ++k)
#pragma unroll
            for (int r = 0; r < 16; ++r) S.acc[k][r][lane] = 0.f;
        float C[4][NCH][4];
#pragma unroll
        for (int mb = 0; mb < 4; ++mb)
#pragma unroll
            for (int ch = 0; ch < NCH; ++ch)
#pragma unroll
                for (int i = 0; i < 4; ++i) C[mb][ch][i] = 0.f;
        float tn_hi = 0.f, tn_lo = 0.f, th_hi = 0.f, th_lo = 0.f;  // this lane's pairs' totals

        // adds the fragments into the lane's double-float sums and clears them
        auto flush = [&]() {
#pragma unroll
            for (int mb = 0; mb < 4; ++mb)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 2 * (2 * mb + (i >> 1)) + (i & 1);  // 2 y + dz
                    float hi = S.acc[0][r][lane], lo = S.acc[1][r][lane];
                    two_sum_acc(hi, lo, C[mb][0][i]);
                    S.acc[0][r][lane] = hi;
                    S.acc[1][r][lane] = lo;
                    C[mb][0][i] = 0.f;
                    if constexpr (NCH > 1) {
                        hi = S.acc[4][r][lane]; lo = S.acc[5][r][lane];
                        two_sum_acc(hi, lo, C[mb][1][i]);
                        S.acc[4][r][lane] = hi; S.acc[5][r][lane] = lo;
                        hi = S.acc[2][r][lane]; lo = S.acc[3][r][lane];
                        two_sum_acc(hi, lo, C[mb][2][i]);
                        S.acc[2][r][lane] = hi; S.acc[3][r][lane] = lo;
#pragma unroll
                        for (int d = 0; d < 3; ++d)
                            S.acc[6 + d][r][lane] = __fadd_rn(S.acc[6 + d][r][lane], C[mb][3 + d][i]);
#pragma unroll
                        for (int ch = 1; ch < NCH; ++ch) C[mb][ch][i] = 0.f;
                    }
                }
        };

        int since_flush = 0;
        for (int c0 = j0; c0 < j1; c0 += 32) {
            // ---- setup: one pair per lane: its image's cell range, 1-D weights
            // (zero outside the range), channel values and FP64 mass; info =
            // the y rows it touches (bits 0-7) and whether it deposits into the
            // n, c, v channels (INFO_MAIN) or the halo channel (INFO_HALO) ----
            uint32_t info = 0;
            {
                const int j = c0 + lane;
                float* wl = S.w[lane];
                float vals[NCH == 1 ? 1 : 6];
#pragma unroll
                for (int k = 0; k < (NCH == 1 ? 1 : 6); ++k) vals[k] = 0.f;
#pragma unroll
                for (int k = 0; k < 3 * TS; ++k) wl[k] = 0.f;
                if (j < j1) {
                    const int i = pvals[j];
                    const int combo = P.periodic ? (int)(pkeys[j] & ((1u << IMG_BITS) - 1u)) : 0;
                    const int dk[3] = {combo % 3, (combo / 3) % 3, combo / 9};
                    float4 A, B, Cc, D;
                    load_dep_rec(rec, i, P.boxsize, P.rbox, A, B, Cc, D);
                    const float xs[3] = {A.x, A.y, A.z};
                    const float lo[3] = {B.x, B.y, B.z};
                    const float hi[3] = {Cc.x, Cc.y, Cc.z};
                    const float hinv = A.w;
                    float mh = 1.0f, ml = 0.0f;  // product of the three 1-D sums (double-float)
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const AxisRange ar = axis_range(lo[a], hi[a], J, nc, periodic);
                        const int k = ar.k_lo + dk[a];
                        const int sh = k * nc + geo.O[a];
                        const int r0 = max(ar.left - sh, 0), r1 = min(ar.right - sh, geo.E[a]);
                        // cell t covers [fi*dx, (fi+1)*dx] with fi = t + sh (see k_deposit_items)
                        float fi = (float)(r0 + sh);
                        float e0 = __fmul_rn(__fmaf_rn(fi, J.dx, -xs[a]), hinv);
                        float sh_ = 0.f, sl_ = 0.f;
                        for (int c = r0; c < r1; ++c) {
                            fi = __fadd_rn(fi, 1.0f);
                            const float e1 = __fmul_rn(__fmaf_rn(fi, J.dx, -xs[a]), hinv);
                            const float wv = tent_integral_rn(e0, e1);
                            wl[a * TS + c] = wv;
                            two_sum_acc(sh_, sl_, wv);
                            e0 = e1;
                        }
                        if (a == 0) { mh = sh_; ml = sl_; }
                        else df_mul_df(mh, ml, sh_, sl_);
                        if (a == 1 && r1 > r0) info = ((1u << r1) - 1u) & ~((1u << r0) - 1u);
                    }
                    const bool halo = (__float_as_int(D.z) & FLAG_HALO) != 0;
                    if (info) info |= halo ? INFO_HALO : INFO_MAIN;
                    if (!halo) {
                        vals[0] = 1.0f;
                        if constexpr (NCH > 1) {
                            vals[2] = B.w;   // dens
                            vals[3] = Cc.w;  // vx
                            vals[4] = D.x;   // vy
                            vals[5] = D.y;   // vz
                        }
                        two_sum_acc(tn_hi, tn_lo, mh);
                        tn_lo = __fadd_rn(tn_lo, ml);
                    } else {
                        if constexpr (NCH > 1) vals[1] = 1.0f;
                        two_sum_acc(th_hi, th_lo, mh);
                        th_lo = __fadd_rn(th_lo, ml);
                    }
                }
#pragma unroll
                for (int k = 0; k < (NCH == 1 ? 1 : 6); ++k) S.v[lane][k] = vals[k];
            }
            __syncwarp();
            // ---- K steps of 8 pairs: pairs 8s + t (A) and 8s + t + 4 (B) for this lane ----
            const int cnt = min(32, j1 - c0);
            for (int s8 = 0; s8 < cnt; s8 += 8) {
                // the rows and channels the step's 8 pairs touch (warp-uniform);
                // the products of the others are exact zeros and are skipped
                const uint32_t kinfo =
                    __reduce_or_sync(FULLM, (lane >= s8 && lane < s8 + 8) ? info : 0u);
                const float* wa = S.w[s8 + t];
                const float* wb = S.w[s8 + t + 4];
                const float xa = wa[g], xb = wb[g];
                const float za = wa[2 * TS + g], zb = wb[2 * TS + g];
                uint32_t bh[NCH][2], bl[NCH][2];
#pragma unroll
                for (int ch = 0; ch < NCH; ++ch) {
                    if (!(kinfo & (ch == 1 && NCH > 1 ? INFO_HALO : INFO_MAIN))) continue;
                    tf32_split(__fmul_rn(za, S.v[s8 + t][ch]), bh[ch][0], bl[ch][0]);
                    tf32_split(__fmul_rn(zb, S.v[s8 + t + 4][ch]), bh[ch][1], bl[ch][1]);
                }
#pragma unroll
                for (int mb = 0; mb < 4; ++mb) {
                    if (!(kinfo & (3u << (2 * mb)))) continue;
                    uint32_t ah[4], al[4];
                    tf32_split(__fmul_rn(xa, wa[TS + 2 * mb]), ah[0], al[0]);
                    tf32_split(__fmul_rn(xa, wa[TS + 2 * mb + 1]), ah[1], al[1]);
                    tf32_split(__fmul_rn(xb, wb[TS + 2 * mb]), ah[2], al[2]);
                    tf32_split(__fmul_rn(xb, wb[TS + 2 * mb + 1]), ah[3], al[3]);
#pragma unroll
                    for (int ch = 0; ch < NCH; ++ch) {
                        if (!(kinfo & (ch == 1 && NCH > 1 ? INFO_HALO : INFO_MAIN))) continue;
                        mma_tf32(C[mb][ch], al, bh[ch][0], bh[ch][1]);
                        mma_tf32(C[mb][ch], ah, bl[ch][0], bl[ch][1]);
                        mma_tf32(C[mb][ch], ah, bh[ch][0], bh[ch][1]);
                    }
                }
            }
            since_flush += 32;
            if (since_flush >= MMA_FLUSH) {
                flush();
                since_flush = 0;
            }
            __syncwarp();  // the next chunk's setup overwrites S.w and S.v
        }
        if (since_flush > 0) flush();

        // ---- this item's FP64 mass, then the tile (final) or the partial tile ----
        double sn = (double)tn_hi + (double)tn_lo, shl = (double)th_hi + (double)th_lo;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sn += __shfl_down_sync(FULLM, sn, o);
            shl += __shfl_down_sync(FULLM, shl, o);
        }
        if (nseg > 1) {
            float* pt = partial + (size_t)item * TC * PW;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int y = r >> 1, z = 2 * t + (r & 1);
                const int e = (z * TS + y) * TS + g;
                pt[e] = S.acc[0][r][lane];
                pt[TC + e] = S.acc[1][r][lane];
                if constexpr (NCH > 1) {
                    pt[2 * TC + e] = S.acc[2][r][lane];
                    pt[3 * TC + e] = S.acc[3][r][lane];
                    pt[4 * TC + e] = S.acc[6][r][lane];
                    pt[5 * TC + e] = S.acc[7][r][lane];
                    pt[6 * TC + e] = S.acc[8][r][lane];
                    pt[7 * TC + e] = S.acc[4][r][lane];
                    pt[8 * TC + e] = S.acc[5][r][lane];
                }
            }
            if (lane == 0) {
                item_tot[2 * item] = sn;
                item_tot[2 * item + 1] = shl;
            }
        } else {
            const size_t nmesh = (size_t)nc * nc * nc;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int y = r >> 1, z = 2 * t + (r & 1);
                if (g >= geo.E[0] || y >= geo.E[1] || z >= geo.E[2]) continue;
                const size_t idx = ((size_t)(geo.O[2] + z) * nc + (geo.O[1] + y)) * nc + (geo.O[0] + g);
                J.mesh[idx] = __fadd_rn(S.acc[0][r][lane], S.acc[1][r][lane]);
                if constexpr (NCH > 1) {
                    J.mesh[nmesh + idx] = __fadd_rn(S.acc[4][r][lane], S.acc[5][r][lane]);
                    J.mesh[2 * nmesh + idx] = __fadd_rn(S.acc[2][r][lane], S.acc[3][r][lane]);
                    J.mesh[3 * nmesh + 3 * idx] = S.acc[6][r][lane];
                    J.mesh[3 * nmesh + 3 * idx + 1] = S.acc[7][r][lane];
                    J.mesh[3 * nmesh + 3 * idx + 2] = S.acc[8][r][lane];
                }
            }
            if (lane == 0) {
                J.partial[2 * geo.local] = sn;
                J.partial[2 * geo.local + 1] = shl;
            }
        }
        __syncwarp();  // the next item clears the sums
    }
}

// The same GEMM with the two warps of a CTA sharing one item: both warps set up
// a chunk of 64 pairs (one pair per thread) in the CTA's staging, then each
// warp runs the K steps for its own half of the tile's y rows (two row blocks,
// 12 fragments) and keeps the double-float sums of its own 8 cells per lane.
// Per CTA 27 KB of shared memory and per thread about half the fragments, so
// about twice as many warps stay resident as with one warp per item.
constexpr int MMA2_CHUNK = 64;  // pairs set up per chunk (one per thread)

template <int NCH>
struct Mma2Cta {
    float acc[2][NCH == 1 ? 2 : 9][8][32];  // [warp][word][2 (y - 4 warp) + dz][lane]
    float w[MMA2_CHUNK][WROW];
    float v[MMA2_CHUNK][NCH == 1 ? 1 : 8];
    uint32_t info[MMA2_CHUNK];
    double tot[2][2];   // per warp: n and halo mass of the item
    int item, tile;
};

template <int NCH>
__global__ void __launch_bounds__(64)
k_deposit_mma2(const float4* __restrict__ rec, DepositParams P, int total_tiles,
               const uint32_t* __restrict__ item_off, const uint32_t* __restrict__ tstart,
               const uint32_t* __restrict__ tcount, const uint32_t* __restrict__ pkeys,
               const int* __restrict__ pvals, float* __restrict__ partial,
               double* __restrict__ item_tot, int* __restrict__ next_item)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NW = NCH == 1 ? 2 : 9;
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    Mma2Cta<NCH>& S = *reinterpret_cast<Mma2Cta<NCH>*>(smem_raw);
    float(*acc)[8][32] = S.acc[wp];
    const bool periodic = P.periodic != 0;
    const uint32_t total_items = item_off[total_tiles];

    for (;;) {
        if (tid == 0) {
            const int it = atomicAdd(next_item, 1);
            S.item = it;
            S.tile = (uint32_t)it < total_items ? upper_index(item_off, total_tiles + 1, (uint32_t)it) : -1;
        }
        __syncthreads();
        const int item = S.item, slot = S.tile;  // items are numbered in slot order
        if ((uint32_t)item >= total_items) break;
        const int tile = P.order ? (int)P.order[slot] : slot;
        const TileGeo geo = tile_geo(P, tile);
        const MeshJob& J = P.job[geo.job];
        const int nc = geo.nc;
        const int seg = item - (int)item_off[slot];
        const int nseg = (int)(item_off[slot + 1] - item_off[slot]);
        const int j0 = (int)tstart[tile] + seg * P.seg;
        const int j1 = (int)tstart[tile] + min((int)tcount[tile], (seg + 1) * P.seg);

#pragma unroll
        for (int k = 0; k < NW; ++k)
#pragma unroll
            for (int r = 0; r < 8; ++r) acc[k][r][lane] = 0.f;
        float C[2][NCH][4];
#pragma unroll
        for (int mb = 0; mb < 2; ++mb)
#pragma unroll
            for (int ch = 0; ch < NCH; ++ch)
#pragma unroll
                for (int i = 0; i < 4; ++i) C[mb][ch][i] = 0.f;
        float tn_hi = 0.f, tn_lo = 0.f, th_hi = 0.f, th_lo = 0.f;

        for (int c0 = j0; c0 < j1; c0 += MMA2_CHUNK) {
            // ---- setup: one pair per thread (as in k_deposit_mma) ----
            {
                const int j = c0 + tid;
                float* wl = S.w[tid];
                float vals[NCH == 1 ? 1 : 6];
#pragma unroll
                for (int k = 0; k < (NCH == 1 ? 1 : 6); ++k) vals[k] = 0.f;
#pragma unroll
                for (int k = 0; k < 3 * TS; ++k) wl[k] = 0.f;
                uint32_t info = 0;
                if (j < j1) {
                    const int i = pvals[j];
                    const int combo = P.periodic ? (int)(pkeys[j] & ((1u << IMG_BITS) - 1u)) : 0;
                    const int dk[3] = {combo % 3, (combo / 3) % 3, combo / 9};
                    float4 A, B, Cc, D;
                    load_dep_rec(rec, i, P.boxsize, P.rbox, A, B, Cc, D);
                    const float xs[3] = {A.x, A.y, A.z};
                    const float lo[3] = {B.x, B.y, B.z};
                    const float hi[3] = {Cc.x, Cc.y, Cc.z};
                    const float hinv = A.w;
                    float mh = 1.0f, ml = 0.0f;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const AxisRange ar = axis_range(lo[a], hi[a], J, nc, periodic);
                        const int k = ar.k_lo + dk[a];
                        const int sh = k * nc + geo.O[a];
                        const int r0 = max(ar.left - sh, 0), r1 = min(ar.right - sh, geo.E[a]);
                        float fi = (float)(r0 + sh);
                        float e0 = __fmul_rn(__fmaf_rn(fi, J.dx, -xs[a]), hinv);
                        float sh_ = 0.f, sl_ = 0.f;
                        for (int c = r0; c < r1; ++c) {
                            fi = __fadd_rn(fi, 1.0f);
                            const float e1 = __fmul_rn(__fmaf_rn(fi, J.dx, -xs[a]), hinv);
                            const float wv = tent_integral_rn(e0, e1);
                            wl[a * TS + c] = wv;
                            two_sum_acc(sh_, sl_, wv);
                            e0 = e1;
                        }
                        if (a == 0) { mh = sh_; ml = sl_; }
                        else df_mul_df(mh, ml, sh_, sl_);
                        if (a == 1 && r1 > r0) info = ((1u << r1) - 1u) & ~((1u << r0) - 1u);
                    }
                    const bool halo = (__float_as_int(D.z) & FLAG_HALO) != 0;
                    if (info) info |= halo ? INFO_HALO : INFO_MAIN;
                    if (!halo) {
                        vals[0] = 1.0f;
                        if constexpr (NCH > 1) {
                            vals[2] = B.w;
                            vals[3] = Cc.w;
                            vals[4] = D.x;
                            vals[5] = D.y;
                        }
                        two_sum_acc(tn_hi, tn_lo, mh);
                        tn_lo = __fadd_rn(tn_lo, ml);
                    } else {
                        if constexpr (NCH > 1) vals[1] = 1.0f;
                        two_sum_acc(th_hi, th_lo, mh);
                        th_lo = __fadd_rn(th_lo, ml);
                    }
                }
#pragma unroll
                for (int k = 0; k < (NCH == 1 ? 1 : 6); ++k) S.v[tid][k] = vals[k];
                S.info[tid] = info;
            }
            __syncthreads();
            // ---- K steps over the chunk, this warp's row blocks 2 wp and 2 wp + 1 ----
            const int cnt = min(MMA2_CHUNK, j1 - c0);
            for (int s8 = 0; s8 < cnt; s8 += 8) {
                const uint32_t kinfo = __reduce_or_sync(FULLM, S.info[s8 + (lane & 7)]);
                const uint32_t rows = 0xfu << (4 * wp);  // the y rows of this warp
                if (!(kinfo & rows)) continue;
                const float* wa = S.w[s8 + t];
                const float* wb = S.w[s8 + t + 4];
                const float xa = wa[g], xb = wb[g];
                const float za = wa[2 * TS + g], zb = wb[2 * TS + g];
                // the channels fed by main particles (n, c, v) and by halo
                // particles (halo) are tested once each, and within a group the
                // three passes run pass by pass over its channels, so the
                // independent accumulation chains interleave
                const bool k_main = (kinfo & INFO_MAIN) != 0;
                const bool k_halo = NCH > 1 && (kinfo & INFO_HALO) != 0;
                uint32_t bh[NCH][2], bl[NCH][2];
                if (k_main) {
#pragma unroll
                    for (int ch = 0; ch < NCH; ++ch) {
                        if (NCH > 1 && ch == 1) continue;
                        tf32_split(__fmul_rn(za, S.v[s8 + t][ch]), bh[ch][0], bl[ch][0]);
                        tf32_split(__fmul_rn(zb, S.v[s8 + t + 4][ch]), bh[ch][1], bl[ch][1]);
                    }
                }
                if (k_halo) {
                    tf32_split(__fmul_rn(za, S.v[s8 + t][1]), bh[1][0], bl[1][0]);
                    tf32_split(__fmul_rn(zb, S.v[s8 + t + 4][1]), bh[1][1], bl[1][1]);
                }
                // the warp's row blocks this K step touches, both in one block
                // of code when both do (twice the independent chains)
                auto blocks = [&](auto use0, auto use1) {
                    constexpr bool U[2] = {decltype(use0)::value, decltype(use1)::value};
                    uint32_t ah[2][4], al[2][4];
#pragma unroll
                    for (int m = 0; m < 2; ++m) {
                        if (!U[m]) continue;
                        const int mb = 2 * wp + m;
                        tf32_split(__fmul_rn(xa, wa[TS + 2 * mb]), ah[m][0], al[m][0]);
                        tf32_split(__fmul_rn(xa, wa[TS + 2 * mb + 1]), ah[m][1], al[m][1]);
                        tf32_split(__fmul_rn(xb, wb[TS + 2 * mb]), ah[m][2], al[m][2]);
                        tf32_split(__fmul_rn(xb, wb[TS + 2 * mb + 1]), ah[m][3], al[m][3]);
                    }
                    if (k_main) {
#pragma unroll
                        for (int m = 0; m < 2; ++m)
#pragma unroll
                            for (int ch = 0; ch < NCH; ++ch)
                                if (U[m] && !(NCH > 1 && ch == 1))
                                    mma_tf32(C[m][ch], al[m], bh[ch][0], bh[ch][1]);
#pragma unroll
                        for (int m = 0; m < 2; ++m)
#pragma unroll
                            for (int ch = 0; ch < NCH; ++ch)
                                if (U[m] && !(NCH > 1 && ch == 1))
                                    mma_tf32(C[m][ch], ah[m], bl[ch][0], bl[ch][1]);
#pragma unroll
                        for (int m = 0; m < 2; ++m)
#pragma unroll
                            for (int ch = 0; ch < NCH; ++ch)
                                if (U[m] && !(NCH > 1 && ch == 1))
                                    mma_tf32(C[m][ch], ah[m], bh[ch][0], bh[ch][1]);
                    }
                    if (k_halo) {
#pragma unroll
                        for (int m = 0; m < 2; ++m)
                            if (U[m]) mma_tf32(C[m][1], al[m], bh[1][0], bh[1][1]);
#pragma unroll
                        for (int m = 0; m < 2; ++m)
                            if (U[m]) mma_tf32(C[m][1], ah[m], bl[1][0], bl[1][1]);
#pragma unroll
                        for (int m = 0; m < 2; ++m)
                            if (U[m]) mma_tf32(C[m][1], ah[m], bh[1][0], bh[1][1]);
                    }
                };
                const bool r0 = (kinfo & (3u << (4 * wp))) != 0;
                const bool r1 = (kinfo & (3u << (4 * wp + 2))) != 0;
                if (r0 && r1) blocks(std::true_type{}, std::true_type{});
                else if (r0) blocks(std::true_type{}, std::false_type{});
                else blocks(std::false_type{}, std::true_type{});
            }
            // ---- flush the fragments into the lane's sums (every chunk of 64 pairs) ----
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 2 * (2 * m + (i >> 1)) + (i & 1);  // 2 (y - 4 wp) + dz
                    float hi = acc[0][r][lane], lo = acc[1][r][lane];
                    two_sum_acc(hi, lo, C[m][0][i]);
                    acc[0][r][lane] = hi;
                    acc[1][r][lane] = lo;
                    C[m][0][i] = 0.f;
                    if constexpr (NCH > 1) {
                        hi = acc[4][r][lane]; lo = acc[5][r][lane];
                        two_sum_acc(hi, lo, C[m][1][i]);
                        acc[4][r][lane] = hi; acc[5][r][lane] = lo;
                        hi = acc[2][r][lane]; lo = acc[3][r][lane];
                        two_sum_acc(hi, lo, C[m][2][i]);
                        acc[2][r][lane] = hi; acc[3][r][lane] = lo;
#pragma unroll
                        for (int d = 0; d < 3; ++d)
                            acc[6 + d][r][lane] = __fadd_rn(acc[6 + d][r][lane], C[m][3 + d][i]);
#pragma unroll
                        for (int ch = 1; ch < NCH; ++ch) C[m][ch][i] = 0.f;
                    }
                }
            __syncthreads();  // the next chunk's setup overwrites the staging
        }

        // ---- the item's FP64 mass (both warps' setup lanes), then the cells ----
        double sn = (double)tn_hi + (double)tn_lo, shl = (double)th_hi + (double)th_lo;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sn += __shfl_down_sync(FULLM, sn, o);
            shl += __shfl_down_sync(FULLM, shl, o);
        }
        if (lane == 0) {
            S.tot[wp][0] = sn;
            S.tot[wp][1] = shl;
        }
        __syncthreads();
        if (tid == 0) {
            sn = S.tot[0][0] + S.tot[1][0];
            shl = S.tot[0][1] + S.tot[1][1];
            if (nseg > 1) {
                item_tot[2 * item] = sn;
                item_tot[2 * item + 1] = shl;
            } else {
                J.partial[2 * geo.local] = sn;
                J.partial[2 * geo.local + 1] = shl;
            }
        }
        if (nseg > 1) {
            float* pt = partial + (size_t)item * TC * PW;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int y = 4 * wp + (r >> 1), z = 2 * t + (r & 1);
                const int e = (z * TS + y) * TS + g;
                pt[e] = acc[0][r][lane];
                pt[TC + e] = acc[1][r][lane];
                if constexpr (NCH > 1) {
                    pt[2 * TC + e] = acc[2][r][lane];
                    pt[3 * TC + e] = acc[3][r][lane];
                    pt[4 * TC + e] = acc[6][r][lane];
                    pt[5 * TC + e] = acc[7][r][lane];
                    pt[6 * TC + e] = acc[8][r][lane];
                    pt[7 * TC + e] = acc[4][r][lane];
                    pt[8 * TC + e] = acc[5][r][lane];
                }
            }
        } else {
            const size_t nmesh = (size_t)nc * nc * nc;
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int y = 4 * wp + (r >> 1), z = 2 * t + (r & 1);
                if (g >= geo.E[0] || y >= geo.E[1] || z >= geo.E[2]) continue;
                const size_t idx = ((size_t)(geo.O[2] + z) * nc + (geo.O[1] + y)) * nc + (geo.O[0] + g);
                J.mesh[idx] = __fadd_rn(acc[0][r][lane], acc[1][r][lane]);
                if constexpr (NCH > 1) {
                    J.mesh[nmesh + idx] = __fadd_rn(acc[4][r][lane], acc[5][r][lane]);
                    J.mesh[2 * nmesh + idx] = __fadd_rn(acc[2][r][lane], acc[3][r][lane]);
                    J.mesh[3 * nmesh + 3 * idx] = acc[6][r][lane];
                    J.mesh[3 * nmesh + 3 * idx + 1] = acc[7][r][lane];
                    J.mesh[3 * nmesh + 3 * idx + 2] = acc[8][r][lane];
                }
            }
        }
        __syncthreads();  // the next item's fetch overwrites S.item, S.tot
    }
}

// ---------------------------------------------------------------------------
// (5) merge the partial tiles of multi-segment tiles, in segment order
// ---------------------------------------------------------------------------
// item_tot (the tensor-core deposit): the FP64 mass of every item, summed in
// item order; null: the mass is summed from the merged cells
__global__ void __launch_bounds__(DEP_THREADS)
k_merge_tiles(DepositParams P, int total_tiles, const uint32_t* __restrict__ item_off,
              const float* __restrict__ partial, const double* __restrict__ item_tot)
{
    __shared__ double red[2][DEP_THREADS / 32];
    const int tile = blockIdx.x;
    const int slot = P.pos ? (int)P.pos[tile] : tile;
    const int i0 = (int)item_off[slot], i1 = (int)item_off[slot + 1];
    if (i1 - i0 <= 1) return;
    const TileGeo g = tile_geo(P, tile);
    const MeshJob& J = P.job[g.job];
    const int nc = g.nc;
    const size_t nmesh = (size_t)nc * nc * nc;
    const int tid = threadIdx.x;
    double sn = 0.0, sh = 0.0;
    for (int e = tid; e < TC; e += DEP_THREADS) {
        float nh = 0.f, nl = 0.f, ch = 0.f, cl = 0.f, vx = 0.f, vy = 0.f, vz = 0.f, hh = 0.f, hl = 0.f;
        for (int it = i0; it < i1; ++it) {
            const float* pt = partial + (size_t)it * TC * PW;
            two_sum_acc(nh, nl, pt[e]);
            nl = __fadd_rn(nl, pt[TC + e]);
            two_sum_acc(ch, cl, pt[2 * TC + e]);
            cl = __fadd_rn(cl, pt[3 * TC + e]);
            vx = __fadd_rn(vx, pt[4 * TC + e]);
            vy = __fadd_rn(vy, pt[5 * TC + e]);
            vz = __fadd_rn(vz, pt[6 * TC + e]);
            two_sum_acc(hh, hl, pt[7 * TC + e]);
            hl = __fadd_rn(hl, pt[8 * TC + e]);
        }
        const int lz = e / (TS * TS), c = e % (TS * TS);
        const int lx = c % TS, ly = c / TS;
        if (lx >= g.E[0] || ly >= g.E[1] || lz >= g.E[2]) continue;
        const size_t idx = ((size_t)(g.O[2] + lz) * nc + (g.O[1] + ly)) * nc + (g.O[0] + lx);
        sn += (double)nh + (double)nl;
        sh += (double)hh + (double)hl;
        J.mesh[idx] = __fadd_rn(nh, nl);
        if (!P.density_only) {
            J.mesh[nmesh + idx] = __fadd_rn(hh, hl);
            J.mesh[2 * nmesh + idx] = __fadd_rn(ch, cl);
            J.mesh[3 * nmesh + 3 * idx] = vx;
            J.mesh[3 * nmesh + 3 * idx + 1] = vy;
            J.mesh[3 * nmesh + 3 * idx + 2] = vz;
        }
    }
    if (item_tot) {
        if (tid == 0) {
            double a = 0.0, b = 0.0;
            for (int it = i0; it < i1; ++it) {
                a += item_tot[2 * it];
                b += item_tot[2 * it + 1];
            }
            J.partial[2 * g.local] = a;
            J.partial[2 * g.local + 1] = b;
        }
        return;
    }
    block_totals(sn, sh, red, J, g.local, tid);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t deposit_prep_bytes(int n) { return 32 * (size_t)n; }

// bits 0-10 of v spread to every third bit
static uint64_t spread3_11(uint32_t v)
{
    uint64_t r = 0;
    for (int b = 0; b < 11; ++b) r |= (uint64_t)((v >> b) & 1u) << (3 * b);
    return r;
}

void deposit_tile_order(const DepositParams& p, int total_tiles, uint32_t* out)
{
    int ncmax = 1;
    for (int k = 0; k < p.n_jobs; ++k) ncmax = std::max(ncmax, p.job[k].nc);
    std::vector<std::pair<uint64_t, uint32_t>> key((size_t)total_tiles);
    for (int k = 0; k < p.n_jobs; ++k) {
        const MeshJob& J = p.job[k];
        int rank = 0;  // coarser meshes first at the same place
        for (int j = 0; j < p.n_jobs; ++j)
            rank += p.job[j].nc < J.nc || (p.job[j].nc == J.nc && j < k);
        // a tile's lower corner, in tiles of the finest mesh (plus half of one)
        const double ratio = (double)ncmax / (double)J.nc;
        const int nt = J.tiles[0] * J.tiles[1] * J.tiles[2];
        for (int t = 0; t < nt; ++t) {
            const int c[3] = {t % J.tiles[0], (t / J.tiles[0]) % J.tiles[1],
                              t / (J.tiles[0] * J.tiles[1])};
            uint64_t m = 0;
            for (int a = 0; a < 3; ++a)
                m |= spread3_11(std::min(2047u, (uint32_t)(c[a] * ratio + 0.5))) << a;
            key[(size_t)(J.tile_begin + t)] = {(m << 4) | (uint64_t)rank,
                                               (uint32_t)(J.tile_begin + t)};
        }
    }
    std::sort(key.begin(), key.end());
    for (int slot = 0; slot < total_tiles; ++slot) {
        out[slot] = key[(size_t)slot].second;
        out[(size_t)total_tiles + key[(size_t)slot].second] = (uint32_t)slot;
    }
}

size_t deposit_tile_bytes(int total_tiles)
{
    // tstart, tcount, item_off (+1 each) and their scan scratch
    const size_t T1 = (size_t)total_tiles + 1;
    return 4 * T1 * 3 + scan_temp_bytes(T1) + 256;
}

static int key_bits(int total_tiles, int ib)
{
    int b = 0;
    while ((1 << b) < total_tiles) ++b;
    return b + ib;
}

// the default deposit engine: 2 the tensor cores with the two warps of a CTA
// per item, 1 with one warp per item, 0 the CUDA cores; ASG_DEPOSIT=mma2, mma
// or simt selects one (a comparison knob; a context's tuner may choose)
int deposit_default_mma()
{
    static const int m = [] {
        const char* e = std::getenv("ASG_DEPOSIT");
        if (e && std::strcmp(e, "simt") == 0) return 0;
        if (e && std::strcmp(e, "mma") == 0) return 1;
        return 2;  // 15.3 against 15.6 ms (one warp per item) on the 256^3 step
    }();
    return m;
}

// per-item FP64 masses after the partial tiles of deposit_max_items items
static double* deposit_item_totals(float* partial, uint32_t items)
{
    const size_t off = ((size_t)items * TC * PW * sizeof(float) + 15) & ~size_t(15);
    return reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(partial) + off);
}

// a persistent kernel: as many CTAs as fit on every SM at once, its dynamic
// shared memory allowed once per device (function attributes are per device)
template <class... KArgs, class... Args>
static void launch_persistent(void (*kern)(KArgs...), int dev, int sms, int threads, size_t smem,
                              cudaStream_t s, Args... args)
{
    static std::atomic<unsigned long long> attr_set{0};  // one bit per device, per kernel
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        attr_set.fetch_or(bit);
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    kern<<<sms * (per_sm > 0 ? per_sm : 1), threads, smem, s>>>(args...);
}

void launch_deposit_prep(const float4* pos, const float4* vel, const int* igrp, const float* rk,
                         int n, const DepositParams& p, DepositScratch& w, int* err,
                         cudaStream_t s)
{
    const int nb = (n + 255) / 256;
    k_dep_prep<<<nb, 256, 0, s>>>(pos, vel, igrp, rk, n, p, w.rec, err);
    k_pairs<false><<<nb, 256, 0, s>>>(w.rec, n, p, w.pcount, nullptr, nullptr, nullptr, 0u, err);
    cudaMemsetAsync(w.pcount + n, 0, 4, s);
    exclusive_scan_u32(w.pcount, (size_t)n + 1, w.scan_tmp_n, s);
    count_launches(2);
}

void launch_deposit_run(int n, const DepositParams& p, int total_tiles, uint32_t npairs, bool padded,
                        DepositScratch& w, int* err, cudaStream_t s)
{
    const int T = total_tiles;
    const int nb = (n + 255) / 256;
    k_pairs<true><<<nb, 256, 0, s>>>(w.rec, n, p, nullptr, w.pcount, w.keys0, w.vals0, npairs, err);
    count_launches(1);
    if (padded && npairs > 0) {  // npairs is the capacity; the count itself is pcount[n]
        k_pad_pairs<<<(npairs + 255) / 256, 256, 0, s>>>(w.keys0, w.vals0, w.pcount + n, npairs,
                                                          (uint32_t)T << img_bits(p));
        count_launches(1);
    }
    const int cur = radix_sort32(w.keys0, w.vals0, w.keys1, w.vals1, (int)npairs,
                                 key_bits(padded ? T + 1 : T, img_bits(p)), w.sort_tmp, s);
    const uint32_t* keys = cur ? w.keys1 : w.keys0;
    const int* vals = cur ? w.vals1 : w.vals0;
    cudaMemsetAsync(w.tstart, 0, 4 * (size_t)T, s);
    cudaMemsetAsync(w.tcount, 0, 4 * (size_t)T, s);
    if (npairs > 0) {
        k_tile_bounds<<<(npairs + 255) / 256, 256, 0, s>>>(keys, (int)npairs, T, img_bits(p), w.tstart,
                                                           w.tcount);
        count_launches(1);
    }
    k_tile_items<<<(T + 1 + 255) / 256, 256, 0, s>>>(w.tstart, w.tcount, T, p.seg, p.pos, w.item_off);
    exclusive_scan_u32(w.item_off, (size_t)T + 1, w.scan_tmp_t, s);
    cudaMemsetAsync(w.next_item, 0, sizeof(int), s);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* item_tot = nullptr;
    if (p.mma == 2) {
        item_tot = deposit_item_totals(w.partial, deposit_max_items(T, npairs, p.seg));
        if (p.density_only)
            launch_persistent(k_deposit_mma2<1>, dev, sms, 64, sizeof(Mma2Cta<1>), s, w.rec, p, T,
                              w.item_off, w.tstart, w.tcount, keys, vals, w.partial, item_tot,
                              w.next_item);
        else
            launch_persistent(k_deposit_mma2<6>, dev, sms, 64, sizeof(Mma2Cta<6>), s, w.rec, p, T,
                              w.item_off, w.tstart, w.tcount, keys, vals, w.partial, item_tot,
                              w.next_item);
    } else if (p.mma) {
        item_tot = deposit_item_totals(w.partial, deposit_max_items(T, npairs, p.seg));
        if (p.density_only)
            launch_persistent(k_deposit_mma<1>, dev, sms, 32 * MMA_WARPS,
                              MMA_WARPS * sizeof(MmaWarp<1>), s, w.rec, p, T, w.item_off, w.tstart,
                              w.tcount, keys, vals, w.partial, item_tot, w.next_item);
        else
            launch_persistent(k_deposit_mma<6>, dev, sms, 32 * MMA_WARPS,
                              MMA_WARPS * sizeof(MmaWarp<6>), s, w.rec, p, T, w.item_off, w.tstart,
                              w.tcount, keys, vals, w.partial, item_tot, w.next_item);
    } else {
        launch_persistent(k_deposit_items, dev, sms, 32 * DEP_WARPS, DEP_WARPS * sizeof(WarpTile), s,
                          w.rec, p, T, w.item_off, w.tstart, w.tcount, keys, vals, w.partial,
                          w.next_item);
    }
    k_merge_tiles<<<T, DEP_THREADS, 0, s>>>(p, T, w.item_off, w.partial, item_tot);
    count_launches(3);
}

uint32_t deposit_max_items(int total_tiles, uint32_t npairs, int seg)
{
    return (uint32_t)total_tiles + npairs / (uint32_t)(seg > 0 ? seg : SEG_DEFAULT) + 1;
}

int deposit_default_seg() { return SEG_DEFAULT; }

// partial tiles of multi-item tiles, then each item's FP64 mass (2 doubles)
size_t deposit_partial_bytes(uint32_t items)
{
    return (((size_t)items * TC * PW * sizeof(float) + 15) & ~size_t(15)) + 16 * (size_t)items;
}

__global__ void k_reduce_partials(const double* __restrict__ partial, int ntiles, double* out2)
{
    __shared__ double r[2][256];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < ntiles; i += blockDim.x) {
        a += partial[2 * i];
        b += partial[2 * i + 1];
    }
    r[0][threadIdx.x] = a;
    r[1][threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            r[0][threadIdx.x] += r[0][threadIdx.x + o];
            r[1][threadIdx.x] += r[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out2[0] = r[0][0];
        out2[1] = r[1][0];
    }
}

void launch_reduce_partials(const double* partial, int ntiles, double* out2, cudaStream_t s)
{
    k_reduce_partials<<<1, 256, 0, s>>>(partial, ntiles, out2);
    count_launches(1);
}

// write_mesh_separate normalisation (coarse_mesh.cpp:158-171), in place
__global__ void k_normalise(float* __restrict__ mesh, size_t nmesh, float vol)
{
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nmesh) return;
    float* n = mesh;
    float* halo = mesh + nmesh;
    float* c = halo + nmesh;
    float* v = c + nmesh;
    const float nj = n[j];
    if (nj > 0.0f) {
        c[j] = __fmul_rn(c[j], __fdiv_rn(vol, __fmul_rn(nj, nj)));
        v[3 * j] = __fdiv_rn(v[3 * j], nj);
        v[3 * j + 1] = __fdiv_rn(v[3 * j + 1], nj);
        v[3 * j + 2] = __fdiv_rn(v[3 * j + 2], nj);
    } else {
        c[j] = 0.0f;
        v[3 * j] = v[3 * j + 1] = v[3 * j + 2] = 0.0f;
    }
    n[j] = __fmul_rn(nj, 8.0f);
    halo[j] = __fmul_rn(halo[j], 8.0f);
}

void launch_normalise(float* mesh, int nc, float vol, cudaStream_t s)
{
    const size_t nmesh = (size_t)nc * nc * nc;
    k_normalise<<<(unsigned)((nmesh + 255) / 256), 256, 0, s>>>(mesh, nmesh, vol);
    count_launches(1);
}

}  // namespace asg
