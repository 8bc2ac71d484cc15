// asg_deposit.cu -- adaptive kernel deposit onto coarse meshes
// (assign_on_mesh, coarse_mesh.cpp:45-127; the periodic assign_on_global_mesh,
// global_mesh.cpp:25-123; the n-only assign_on_density_mesh, :212-269), the
// FP64 mass totals (mesh_total / check_total_mass, coarse_mesh.cpp:35-43,
// clumping_tree_main.cpp:578-600) and the write_mesh_separate normalisation
// (coarse_mesh.cpp:158-171).
//
// Per particle and per cell the weight is bit-identical to the reference:
// cell range [left, right) per axis from the reference's float expression,
// k = ker_integ(s1, s1 + ds) with s1 = (i*dx - x)*hinv, ker3 = (k0*k1)*k2.
//
// Deterministic gather, no atomics on the mesh.  The mesh is cut into 8^3-cell
// tiles.  (1) One warp per tile walks the particle radix tree (node boxes
// expanded by the particles' smoothing lengths) and lists, in depth-first
// order, the buckets whose cell ranges can touch the tile.  (2) Each tile's
// candidate list is cut into segments of SEG particles; a persistent kernel
// deposits one (tile, segment) per CTA into a shared-memory tile: warp w owns
// z-layer w and adds one particle after another, so every cell sums its
// contributions in list order.  (3) Tiles with several segments merge their
// partial tiles in segment order.  n, c and halo are double-float (two-sum)
// sums, so the tile totals reproduce the FP64 sum of the float weights.
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

constexpr int TS = 8;              // tile edge in cells
constexpr int TC = TS * TS * TS;   // cells per tile
constexpr int DEP_THREADS = 256;   // 8 warps: warp w <-> z-layer w
constexpr int CH = 64;             // particles per processing chunk
constexpr int SEG = 2048;          // particles per work item
constexpr int PW = 9;              // partial words per cell
constexpr unsigned FULLM = 0xffffffffu;

// ---------------------------------------------------------------------------
// tile geometry and the node / particle cell ranges
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

// conservative cell interval [a, b) of an expanded box along one axis
__device__ __forceinline__ void node_cells(float lo, float hi, float boxsize, float ncf, int& a,
                                           int& b)
{
    const float fa = floorf(lo / boxsize * ncf) - 1.0f;
    const float fb = floorf(hi / boxsize * ncf) + 2.0f;
    a = (int)fmaxf(fminf(fa, 1.0e9f), -1.0e9f);
    b = (int)fmaxf(fminf(fb, 1.0e9f), -1.0e9f);
}

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

__device__ __forceinline__ bool cells_hit(int a, int b, int X0, int X1, int nc, bool periodic)
{
    if (!periodic) return a < X1 && b > X0;
    if (b - a >= nc) return true;
    const int k = floor_div(a, nc);
    const int a2 = a - k * nc, b2 = b - k * nc;  // a2 in [0, nc)
    return (a2 < X1 && b2 > X0) || (b2 - nc > X0);
}

__device__ __forceinline__ bool node_hits_tile(float4 lo, float4 hi, const DepositParams& P,
                                               float ncf, const TileGeo& g)
{
    const bool per = P.periodic != 0;
    if (per) {
        lo.x += P.offset[0]; lo.y += P.offset[1]; lo.z += P.offset[2];
        hi.x += P.offset[0]; hi.y += P.offset[1]; hi.z += P.offset[2];
    }
    int a0, b0, a1, b1, a2, b2;
    node_cells(lo.x, hi.x, P.boxsize, ncf, a0, b0);
    node_cells(lo.y, hi.y, P.boxsize, ncf, a1, b1);
    node_cells(lo.z, hi.z, P.boxsize, ncf, a2, b2);
    return cells_hit(a0, b0, g.O[0], g.O[0] + g.E[0], g.nc, per) &&
           cells_hit(a1, b1, g.O[1], g.O[1] + g.E[1], g.nc, per) &&
           cells_hit(a2, b2, g.O[2], g.O[2] + g.E[2], g.nc, per);
}

// ---------------------------------------------------------------------------
// (1) candidate lists: one warp per tile, depth-first, left subtree first
// ---------------------------------------------------------------------------
constexpr int LIST_WARPS = 4;
constexpr int LIST_STACK = 512;  // per-warp node stack of the lane-parallel walk

template <bool FILL>
__global__ void __launch_bounds__(LIST_WARPS * 32)
k_tile_lists(const float4* __restrict__ pos, const float* __restrict__ rk, TreeView t,
             DepositParams P, int total_tiles, uint32_t* __restrict__ nranges,
             uint32_t* __restrict__ nparts, const uint32_t* __restrict__ range_off,
             int4* __restrict__ ranges, int* next_item, int* err)
{
    __shared__ int stk[LIST_WARPS][LIST_STACK];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x * LIST_WARPS + warp;
    if (tile >= total_tiles) return;
    const TileGeo g = tile_geo(P, tile);
    const float ncf = P.job[g.job].ncf;
    int* st = stk[warp];
    if (lane == 0) st[0] = tree_root(t.n);
    int sp = 1;
    uint32_t nr = 0, np = 0;
    const uint32_t base = FILL ? range_off[tile] : 0u;
    bool ovf = false;
    const unsigned lt = lanemask_lt();
    __syncwarp();
    // each round the lanes test up to 32 nodes from the top of the stack; hit
    // buckets are listed in lane order, hit inner nodes push their children in
    // lane order (the order depends only on the data: count and fill agree)
    while (sp > 0) {
        const int take = (sp + 64 <= LIST_STACK) ? min(sp, 32) : 1;
        const bool act = lane < take;
        const int node = act ? st[sp - take + lane] : 0;
        sp -= take;
        __syncwarp();
        bool hit = false, bucket = false;
        int first = 0, last = -1, c0 = 0, c1 = 0;
        if (act) {
            float4 lo, hi;
            if (node < 0) {
                const int i = ~node;
                const float4 p = pos[i];
                const float h = __fmul_ru(rk[i], 1.000001f);
                lo = make_float4(__fsub_rd(p.x, h), __fsub_rd(p.y, h), __fsub_rd(p.z, h), 0.f);
                hi = make_float4(__fadd_ru(p.x, h), __fadd_ru(p.y, h), __fadd_ru(p.z, h), 0.f);
                first = last = i;
                bucket = true;
            } else {
                const int4 m = t.meta[node];
                lo = t.elo[node];
                hi = t.ehi[node];
                first = m.z;
                last = m.w;
                c0 = m.x;
                c1 = m.y;
                bucket = (m.w - m.z + 1) <= LEAF_MAX;
            }
            hit = node_hits_tile(lo, hi, P, ncf, g);
        }
        const unsigned bmask = __ballot_sync(FULLM, hit && bucket);
        const unsigned imask = __ballot_sync(FULLM, hit && !bucket);
        {
            // exclusive prefix of bucket sizes over lanes (0 for non-buckets)
            int cnt = (hit && bucket) ? (last - first + 1) : 0;
            int inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULLM, inc, o);
                if (lane >= o) inc += y;
            }
            const int tot = __shfl_sync(FULLM, inc, 31);
            if (hit && bucket) {
                const int slot = __popc(bmask & lt);
                if (FILL) ranges[base + nr + slot] = make_int4(first, last, (int)np + inc - cnt, 0);
            }
            nr += __popc(bmask);
            np += (uint32_t)tot;
        }
        const int ni = __popc(imask);
        if (sp + 2 * ni > LIST_STACK) { ovf = true; break; }
        if (hit && !bucket) {
            // the lowest hit lane ends on top: push in reverse lane order
            const int r = ni - 1 - __popc(imask & lt);
            st[sp + 2 * r] = c1;
            st[sp + 2 * r + 1] = c0;
        }
        sp += 2 * ni;
        __syncwarp();
    }
    if (lane == 0) {
        if (ovf) atomicOr(err, ERR_STACK);
        if (!FILL) {
            nranges[tile] = nr;
            nparts[tile] = np;
            // next_item[2..3] accumulate the candidate particle-tile pairs (statistics)
            atomicAdd(reinterpret_cast<unsigned long long*>(next_item + 2), (unsigned long long)np);
        }
    }
}

// number of SEG-particle work items per tile (at least one, so every tile is written)
__global__ void k_tile_items(const uint32_t* __restrict__ nparts, int total_tiles,
                             uint32_t* __restrict__ nitems)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total_tiles) nitems[i] = max(1u, (nparts[i] + SEG - 1) / SEG);
    if (i == total_tiles) nitems[i] = 0u;
}

// ---------------------------------------------------------------------------
// (2) persistent deposit of (tile, segment) work items
// ---------------------------------------------------------------------------
struct DepShared {
    float4 accA[TS][TS * TS];  // n_hi, n_lo, c_hi, c_lo
    float4 accB[TS][TS * TS];  // vx, vy, vz, halo_hi
    float accC[TS][TS * TS];   // halo_lo
    int item, tile;
    int ok[CH];
    int lohi[CH][6];    // cell ranges [left, right) per axis (unwrapped when periodic)
    int kmin[CH][3];    // first mesh image per axis (periodic)
    int nk[CH][3];      // images per axis
    float px[CH][3];    // position (offset applied for the periodic mesh)
    float ph[CH][2];    // hinv, ds
    float4 val[CH];     // dens, vx, vy, vz
    int halo[CH];
    float w[CH][3][TS]; // 1-D cell weights over the tile's cells, per axis, this image
    double red[2][DEP_THREADS / 32];
};

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

__global__ void __launch_bounds__(DEP_THREADS)
k_deposit_items(const float4* __restrict__ pos, const float4* __restrict__ vel,
                const int* __restrict__ igrp, const float* __restrict__ rk, DepositParams P,
                int total_tiles, const uint32_t* __restrict__ item_off,
                const uint32_t* __restrict__ nparts, const uint32_t* __restrict__ range_off,
                const uint32_t* __restrict__ nranges, const int4* __restrict__ ranges,
                float* __restrict__ partial, int* __restrict__ next_item, int* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DepShared& S = *reinterpret_cast<DepShared*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool periodic = P.periodic != 0;
    const float L = P.boxsize;
    const uint32_t total_items = item_off[total_tiles];

    for (;;) {
        if (tid == 0) {
            const int it = atomicAdd(next_item, 1);
            S.item = it;
            S.tile = (uint32_t)it < total_items ? upper_index(item_off, total_tiles + 1, (uint32_t)it) : -1;
        }
        __syncthreads();
        const int item = S.item, tile = S.tile;
        if ((uint32_t)item >= total_items) break;
        const TileGeo g = tile_geo(P, tile);
        const MeshJob& J = P.job[g.job];
        const int nc = g.nc;
        const int seg = item - (int)item_off[tile];
        const int nseg = (int)(item_off[tile + 1] - item_off[tile]);
        const int p_begin = seg * SEG;
        const int p_end = min((int)nparts[tile], p_begin + SEG);

        for (int e = tid; e < TC; e += DEP_THREADS) {
            (&S.accA[0][0])[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            (&S.accB[0][0])[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            (&S.accC[0][0])[e] = 0.f;
        }
        // the tile's ranges are contiguous from r0; .z is each range's flattened start
        const uint32_t r0 = range_off[tile];
        const int nr = (int)nranges[tile];
        __syncthreads();

        // current range and its first flattened index: the range holding p_begin
        int r = 0;
        {
            int lo = 0, hi = nr - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (ranges[r0 + mid].z <= p_begin) lo = mid; else hi = mid - 1;
            }
            r = lo;
        }
        int r_start = nr > 0 ? ranges[r0 + r].z : 0;
        for (int c0 = p_begin; c0 < p_end; c0 += CH) {
            if (tid < CH) {
                const int p = c0 + tid;
                int ok = 0;
                if (p < p_end) {
                    // walk the tile's ranges to particle p (each thread independently)
                    int rr = r, rs = r_start;
                    for (;;) {
                        const int4 rg = ranges[r0 + rr];
                        const int len = rg.y - rg.x + 1;
                        if (p < rs + len) break;
                        rs += len;
                        ++rr;
                    }
                    const int s = ranges[r0 + rr].x + (p - rs);
                    const float4 q = pos[s];
                    const float h = rk[s];
                    const int to_halo = (P.sign * igrp[s]) > 0;
                    ok = !(P.density_only && to_halo);
                    float x[3] = {q.x, q.y, q.z};
                    if (periodic) {  // global_mesh.cpp:52-61
                        if (q.x < 0.0f || q.x >= L || q.y < 0.0f || q.y >= L || q.z < 0.0f ||
                            q.z >= L)
                            ok = 0;
                        x[0] = __fadd_rn(x[0], P.offset[0]);
                        x[1] = __fadd_rn(x[1], P.offset[1]);
                        x[2] = __fadd_rn(x[2], P.offset[2]);
                    }
                    const float hinv = __fdiv_rn(1.0f, h);
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const float fl = __fmul_rn(__fdiv_rn(__fsub_rn(x[a], h), L), J.ncf);
                        const float fr = __fmul_rn(__fdiv_rn(__fadd_rn(x[a], h), L), J.ncf);
                        int left, right, k0 = 0, nk = 1;
                        if (periodic) {  // global_mesh.cpp:66-69, cells wrap (:85-87)
                            left = (int)floorf(fl);
                            right = 1 + (int)ceilf(fr);
                            // images k with [left-k*nc, right-k*nc) meeting the tile
                            k0 = floor_div(left - g.O[a] - g.E[a], nc) + 1;
                            const int k1 = floor_div(right - g.O[a] - 1, nc);
                            nk = k1 - k0 + 1;
                            if (nk > 3) {
                                atomicOr(err, ERR_RANGE);
                                ok = 0;
                            }
                            if (nk <= 0) ok = 0;
                        } else {  // coarse_mesh.cpp:72-75
                            left = max(0, __float2int_rz(fl));
                            right = min(nc, 1 + __float2int_rz(fr));
                            if (max(left, g.O[a]) >= min(right, g.O[a] + g.E[a])) ok = 0;
                        }
                        S.lohi[tid][2 * a] = left;
                        S.lohi[tid][2 * a + 1] = right;
                        S.kmin[tid][a] = k0;
                        S.nk[tid][a] = nk;
                        S.px[tid][a] = x[a];
                    }
                    S.ph[tid][0] = hinv;
                    S.ph[tid][1] = __fmul_rn(J.dx, hinv);
                    const float4 v = vel[s];
                    S.val[tid] = make_float4(v.w, v.x, v.y, v.z);
                    S.halo[tid] = to_halo;
                }
                S.ok[tid] = ok;
            }
            // advance the shared range cursor past this chunk (thread-uniform)
            {
                const int pe = min(c0 + CH, p_end);
                while (r < nr) {
                    const int4 rg = ranges[r0 + r];
                    const int len = rg.y - rg.x + 1;
                    if (pe < r_start + len) break;
                    r_start += len;
                    ++r;
                }
            }
            __syncthreads();
            const int ncombo = periodic ? 27 : 1;
            for (int combo = 0; combo < ncombo; ++combo) {
                const int dk[3] = {combo % 3, (combo / 3) % 3, combo / 9};
                // 1-D weights of every chunk particle over the tile's cells, this image
                for (int e = tid; e < CH * 3 * TS; e += DEP_THREADS) {
                    const int p = e / (3 * TS), a = (e / TS) % 3, k = e % TS;
                    float w = 0.0f;
                    if (S.ok[p] && k < g.E[a] && dk[a] < S.nk[p][a]) {
                        const int left = S.lohi[p][2 * a], right = S.lohi[p][2 * a + 1];
                        const int ii = g.O[a] + k + (S.kmin[p][a] + dk[a]) * nc;
                        if (ii >= left && ii < right) {
                            const float s1 = __fmul_rn(__fsub_rn(__fmul_rn((float)ii, J.dx), S.px[p][a]),
                                                       S.ph[p][0]);
                            w = ker_integ_rn(s1, __fadd_rn(s1, S.ph[p][1]));
                        }
                    }
                    S.w[p][a][k] = w;
                }
                __syncthreads();
                // warp w deposits every chunk particle that touches z-layer w, in order
                if (warp < g.E[2]) {
                    for (int half = 0; half < CH / 32; ++half) {
                        const int pl = half * 32 + lane;
                        bool mine = false;
                        int rect[6] = {0, 0, 0, 0, 0, 0};
                        if (S.ok[pl] && dk[0] < S.nk[pl][0] && dk[1] < S.nk[pl][1] &&
                            dk[2] < S.nk[pl][2]) {
#pragma unroll
                            for (int a = 0; a < 3; ++a) {
                                const int sh = (S.kmin[pl][a] + dk[a]) * nc + g.O[a];
                                rect[2 * a] = max(S.lohi[pl][2 * a] - sh, 0);
                                rect[2 * a + 1] = min(S.lohi[pl][2 * a + 1] - sh, g.E[a]);
                            }
                            mine = rect[0] < rect[1] && rect[2] < rect[3] && warp >= rect[4] &&
                                   warp < rect[5];
                        }
                        unsigned mask = __ballot_sync(FULLM, mine);
                        const int x0l = rect[0], x1l = rect[1], y0l = rect[2], y1l = rect[3];
                        while (mask) {
                            const int src = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const int p = half * 32 + src;
                            const int x0 = __shfl_sync(FULLM, x0l, src), x1 = __shfl_sync(FULLM, x1l, src);
                            const int y0 = __shfl_sync(FULLM, y0l, src), y1 = __shfl_sync(FULLM, y1l, src);
                            const int nx = x1 - x0;
                            const int ncell = nx * (y1 - y0);
                            const float kz = S.w[p][2][warp];
                            const float4 val = S.val[p];
                            const int hal = S.halo[p];
                            for (int c = lane; c < ncell; c += 32) {
                                const int ix = x0 + c % nx, iy = y0 + c / nx;
                                const float w3 = __fmul_rn(__fmul_rn(S.w[p][0][ix], S.w[p][1][iy]), kz);
                                const int cell = iy * TS + ix;
                                if (!hal) {
                                    float4 A = S.accA[warp][cell];
                                    float4 B = S.accB[warp][cell];
                                    two_sum_acc(A.x, A.y, w3);
                                    const float pr = __fmul_rn(w3, val.x);
                                    const float pe = fmaf(w3, val.x, -pr);
                                    two_sum_acc(A.z, A.w, pr);
                                    A.w = __fadd_rn(A.w, pe);
                                    B.x = fmaf(w3, val.y, B.x);
                                    B.y = fmaf(w3, val.z, B.y);
                                    B.z = fmaf(w3, val.w, B.z);
                                    S.accA[warp][cell] = A;
                                    S.accB[warp][cell] = B;
                                } else {
                                    float hh = S.accB[warp][cell].w, hl = S.accC[warp][cell];
                                    two_sum_acc(hh, hl, w3);
                                    S.accB[warp][cell].w = hh;
                                    S.accC[warp][cell] = hl;
                                }
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }

        // ---- write: final tile when alone, partial tile otherwise ----
        const size_t nmesh = (size_t)nc * nc * nc;
        if (nseg > 1) {
            float* pt = partial + (size_t)item * TC * PW;
            for (int e = tid; e < TC; e += DEP_THREADS) {
                const int lz = e / (TS * TS), c = e % (TS * TS);
                const float4 A = S.accA[lz][c];
                const float4 B = S.accB[lz][c];
                pt[e] = A.x; pt[TC + e] = A.y; pt[2 * TC + e] = A.z; pt[3 * TC + e] = A.w;
                pt[4 * TC + e] = B.x; pt[5 * TC + e] = B.y; pt[6 * TC + e] = B.z;
                pt[7 * TC + e] = B.w; pt[8 * TC + e] = S.accC[lz][c];
            }
        } else {
            double sn = 0.0, sh = 0.0;
            for (int e = tid; e < TC; e += DEP_THREADS) {
                const int lz = e / (TS * TS), c = e % (TS * TS);
                const int lx = c % TS, ly = c / TS;
                if (lx >= g.E[0] || ly >= g.E[1] || lz >= g.E[2]) continue;
                const float4 A = S.accA[lz][c];
                const float4 B = S.accB[lz][c];
                const float hl = S.accC[lz][c];
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
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sn += __shfl_down_sync(FULLM, sn, o);
                sh += __shfl_down_sync(FULLM, sh, o);
            }
            if (lane == 0) {
                S.red[0][warp] = sn;
                S.red[1][warp] = sh;
            }
            __syncthreads();
            if (tid == 0) {
                double a = 0.0, b = 0.0;
                for (int w = 0; w < DEP_THREADS / 32; ++w) {
                    a += S.red[0][w];
                    b += S.red[1][w];
                }
                J.partial[2 * g.local] = a;
                J.partial[2 * g.local + 1] = b;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// (3) merge the partial tiles of multi-segment tiles, in segment order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(DEP_THREADS)
k_merge_tiles(DepositParams P, int total_tiles, const uint32_t* __restrict__ item_off,
              const float* __restrict__ partial)
{
    __shared__ double red[2][DEP_THREADS / 32];
    const int tile = blockIdx.x;
    const int i0 = (int)item_off[tile], i1 = (int)item_off[tile + 1];
    if (i1 - i0 <= 1) return;
    const TileGeo g = tile_geo(P, tile);
    const MeshJob& J = P.job[g.job];
    const int nc = g.nc;
    const size_t nmesh = (size_t)nc * nc * nc;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
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
        J.partial[2 * g.local] = a;
        J.partial[2 * g.local + 1] = b;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t deposit_list_temp_bytes(int total_tiles)
{
    // nranges, nparts, nitems/item_off, range_off (+1 each), scan scratch, counters
    const size_t T = (size_t)total_tiles + 1;
    return 4 * T * 4 + 2 * scan_temp_bytes(T) + 256;
}

int launch_deposit_count(const float4* pos, const float* rk, const TreeView& t,
                         const DepositParams& p, int total_tiles, DepositScratch& w, int* err,
                         cudaStream_t s)
{
    const int T = total_tiles;
    const int lb = (T + LIST_WARPS - 1) / LIST_WARPS;
    cudaMemsetAsync(w.next_item, 0, 16, s);
    k_tile_lists<false><<<lb, LIST_WARPS * 32, 0, s>>>(pos, rk, t, p, T, w.nranges, w.nparts,
                                                       nullptr, nullptr, w.next_item, err);
    // range_off = exclusive scan of nranges; item_off = exclusive scan of items per tile
    cudaMemcpyAsync(w.range_off, w.nranges, 4 * (size_t)T, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(w.range_off + T, 0, 4, s);
    exclusive_scan_u32(w.range_off, (size_t)T + 1, w.scan_tmp, s);
    k_tile_items<<<(T + 1 + 255) / 256, 256, 0, s>>>(w.nparts, T, w.item_off);
    exclusive_scan_u32(w.item_off, (size_t)T + 1, w.scan_tmp, s);
    count_launches(2);
    return 0;
}

void launch_deposit_run(const float4* pos, const float4* vel, const int* igrp, const float* rk,
                        const TreeView& t, const DepositParams& p, int total_tiles,
                        DepositScratch& w, int* err, cudaStream_t s)
{
    const int T = total_tiles;
    const int lb = (T + LIST_WARPS - 1) / LIST_WARPS;
    k_tile_lists<true><<<lb, LIST_WARPS * 32, 0, s>>>(pos, rk, t, p, T, nullptr, nullptr,
                                                      w.range_off, w.ranges, nullptr, err);
    cudaMemsetAsync(w.next_item, 0, sizeof(int), s);
    const size_t smem = sizeof(DepShared);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_deposit_items, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_deposit_items, DEP_THREADS, smem);
    const int grid = sms * (per_sm > 0 ? per_sm : 1);
    k_deposit_items<<<grid, DEP_THREADS, smem, s>>>(pos, vel, igrp, rk, p, T, w.item_off, w.nparts,
                                                    w.range_off, w.nranges, w.ranges, w.partial,
                                                    w.next_item, err);
    k_merge_tiles<<<T, DEP_THREADS, 0, s>>>(p, T, w.item_off, w.partial);
    count_launches(3);
}

size_t deposit_partial_bytes(uint32_t items) { return (size_t)items * TC * PW * sizeof(float); }

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
