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
// Gather, deterministic, no atomics: one CTA owns an 8x8x8 tile of one mesh and
// warp w owns z-layer w of the tile.  Warp 0 walks the particle radix tree
// (node boxes expanded by the particles' smoothing lengths) and lists the
// buckets whose cell ranges can touch the tile; all warps then stream those
// particles in list order.  Each cell is updated by its layer's warp only, one
// particle after another, so every cell sums its contributions in a fixed
// order.  n, c and halo are accumulated as double-float (two-sum), so the tile
// totals reproduce the FP64 sum of the float weights.
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

constexpr int TS = 8;              // tile edge in cells
constexpr int DEP_THREADS = 256;   // 8 warps: warp w <-> z-layer w
constexpr int MAXR = 64;           // bucket ranges listed per round
constexpr int CH = 32;             // particles per processing chunk
constexpr unsigned FULLM = 0xffffffffu;

struct DepShared {
    float4 accA[TS][TS * TS];  // n_hi, n_lo, c_hi, c_lo
    float4 accB[TS][TS * TS];  // vx, vy, vz, halo_hi
    float accC[TS][TS * TS];   // halo_lo
    int stk[STACK_MAX];
    int2 rng[MAXR];
    int rpre[MAXR + 1];
    int nr, sp, done;
    // chunk data
    int ok[CH];
    int rect[CH][6];    // tile-relative [x0,x1) [y0,y1) [z0,z1)
    int lohi[CH][6];    // unclipped/unwrapped cell ranges left/right per axis
    float px[CH][3];    // position (offset applied for the periodic mesh)
    float ph[CH][2];    // hinv, ds
    float4 val[CH];     // dens, vx, vy, vz
    int halo[CH];
    float w[CH][3][TS]; // 1-D cell weights over the tile's cells, per axis
    double red[2][DEP_THREADS / 32];
};

__device__ __forceinline__ int trunc_i(float v) { return __float2int_rz(v); }

// conservative cell interval [a, b) of a node's expanded box along one axis
__device__ __forceinline__ void node_cells(float lo, float hi, float boxsize, float ncf, int& a,
                                           int& b)
{
    const float fa = floorf(lo / boxsize * ncf) - 1.0f;
    const float fb = floorf(hi / boxsize * ncf) + 2.0f;
    a = (int)fmaxf(fminf(fa, 1.0e9f), -1.0e9f);
    b = (int)fmaxf(fminf(fb, 1.0e9f), -1.0e9f);
}

__device__ __forceinline__ bool cells_hit(int a, int b, int X0, int X1, int nc, bool periodic)
{
    if (!periodic) return a < X1 && b > X0;
    if (b - a >= nc) return true;
    int k = a >= 0 ? a / nc : -((-a + nc - 1) / nc);
    const int a2 = a - k * nc, b2 = b - k * nc;  // a2 in [0, nc)
    return (a2 < X1 && b2 > X0) || (b2 - nc > X0);
}

__global__ void __launch_bounds__(DEP_THREADS)
k_deposit(const float4* __restrict__ pos, const float4* __restrict__ vel,
          const int* __restrict__ igrp, const float* __restrict__ rk, TreeView t,
          DepositParams P, int* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DepShared& S = *reinterpret_cast<DepShared*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    int jb = 0;
    while (jb + 1 < P.n_jobs && (int)blockIdx.x >= P.job[jb + 1].tile_begin) ++jb;
    const MeshJob J = P.job[jb];
    const int local = blockIdx.x - J.tile_begin;
    const int nc = J.nc;
    const int tx = local % J.tiles[0];
    const int ty = (local / J.tiles[0]) % J.tiles[1];
    const int tz = local / (J.tiles[0] * J.tiles[1]);
    const int O[3] = {tx * TS, ty * TS, tz * TS};
    const int E[3] = {min(TS, nc - O[0]), min(TS, nc - O[1]), min(TS, nc - O[2])};
    const bool periodic = P.periodic != 0;
    const float L = P.boxsize;

    for (int e = tid; e < TS * TS * TS; e += DEP_THREADS) {
        (&S.accA[0][0])[e] = make_float4(0.f, 0.f, 0.f, 0.f);
        (&S.accB[0][0])[e] = make_float4(0.f, 0.f, 0.f, 0.f);
        (&S.accC[0][0])[e] = 0.f;
    }
    if (tid == 0) {
        S.stk[0] = tree_root(t.n);
        S.sp = 1;
        S.done = 0;
        S.nr = 0;
    }
    __syncthreads();

    for (;;) {
        // ---- phase A: warp 0 lists buckets that can touch the tile ----
        if (warp == 0) {
            int sp = S.sp, nr = 0;
            bool ovf = false;
            while (sp > 0 && nr < MAXR) {
                const int node = S.stk[sp - 1];
                --sp;
                __syncwarp();
                float4 lo, hi;
                int first, last;
                bool bucket;
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
                    bucket = (m.w - m.z + 1) <= LEAF_MAX;
                }
                if (periodic) {
                    lo.x += P.offset[0]; lo.y += P.offset[1]; lo.z += P.offset[2];
                    hi.x += P.offset[0]; hi.y += P.offset[1]; hi.z += P.offset[2];
                }
                int a0, b0, a1, b1, a2, b2;
                node_cells(lo.x, hi.x, L, J.ncf, a0, b0);
                node_cells(lo.y, hi.y, L, J.ncf, a1, b1);
                node_cells(lo.z, hi.z, L, J.ncf, a2, b2);
                const bool hit = cells_hit(a0, b0, O[0], O[0] + E[0], nc, periodic) &&
                                 cells_hit(a1, b1, O[1], O[1] + E[1], nc, periodic) &&
                                 cells_hit(a2, b2, O[2], O[2] + E[2], nc, periodic);
                if (!hit) continue;
                if (bucket) {
                    if (lane == 0) S.rng[nr] = make_int2(first, last);
                    ++nr;
                } else {
                    if (sp + 2 > STACK_MAX) { ovf = true; break; }
                    const int4 m = t.meta[node];
                    if (lane == 0) {
                        S.stk[sp] = m.y;  // left subtree first: input-independent order
                        S.stk[sp + 1] = m.x;
                    }
                    sp += 2;
                }
                __syncwarp();
            }
            if (ovf && lane == 0) atomicOr(err, ERR_STACK);
            if (lane == 0) {
                S.sp = ovf ? 0 : sp;
                S.nr = nr;
                S.done = (ovf || sp == 0) ? 1 : 0;
                int acc = 0;
                for (int r = 0; r < nr; ++r) {
                    S.rpre[r] = acc;
                    acc += S.rng[r].y - S.rng[r].x + 1;
                }
                S.rpre[nr] = acc;
            }
        }
        __syncthreads();
        const int nr = S.nr;
        const int total = S.rpre[nr];

        // ---- phase B: stream the listed particles in chunks of CH ----
        for (int c0 = 0; c0 < total; c0 += CH) {
            if (tid < CH) {
                const int p = c0 + tid;
                int ok = 0;
                if (p < total) {
                    int r = 0;
                    while (S.rpre[r + 1] <= p) ++r;
                    const int s = S.rng[r].x + (p - S.rpre[r]);
                    const float4 q = pos[s];
                    const float h = rk[s];
                    const int to_halo = (P.sign * igrp[s]) > 0;
                    ok = 1;
                    if (P.density_only && to_halo) ok = 0;
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
                        int left, right;
                        const float fl = __fmul_rn(__fdiv_rn(__fsub_rn(x[a], h), L), J.ncf);
                        const float fr = __fmul_rn(__fdiv_rn(__fadd_rn(x[a], h), L), J.ncf);
                        int r0, r1;
                        if (periodic) {  // global_mesh.cpp:66-69
                            left = (int)floorf(fl);
                            right = 1 + (int)ceilf(fr);
                            if (right - left > nc) {
                                atomicOr(err, ERR_RANGE);
                                ok = 0;
                            }
                            r0 = 0;
                            r1 = E[a];
                        } else {  // coarse_mesh.cpp:72-75
                            left = max(0, trunc_i(fl));
                            right = min(nc, 1 + trunc_i(fr));
                            r0 = max(left, O[a]) - O[a];
                            r1 = min(right, O[a] + E[a]) - O[a];
                            if (r0 >= r1) ok = 0;
                        }
                        S.lohi[tid][2 * a] = left;
                        S.lohi[tid][2 * a + 1] = right;
                        S.rect[tid][2 * a] = r0;
                        S.rect[tid][2 * a + 1] = r1;
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
            __syncthreads();
            // 1-D weights of every listed particle over the tile's cells
            for (int e = tid; e < CH * 3 * TS; e += DEP_THREADS) {
                const int p = e / (3 * TS), a = (e / TS) % 3, k = e % TS;
                float w = 0.0f;
                if (S.ok[p] && k < E[a]) {
                    const int left = S.lohi[p][2 * a], right = S.lohi[p][2 * a + 1];
                    int ii = O[a] + k;
                    if (periodic) {  // the image of this cell inside [left, right)
                        int d = (ii - left) % nc;
                        if (d < 0) d += nc;
                        ii = left + d;
                    }
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
            if (warp < E[2]) {
                const int pl = lane;
                const bool mine = S.ok[pl] && warp >= S.rect[pl][4] && warp < S.rect[pl][5];
                unsigned mask = __ballot_sync(FULLM, mine);
                while (mask) {
                    const int p = __ffs(mask) - 1;
                    mask &= mask - 1;
                    const int x0 = S.rect[p][0], x1 = S.rect[p][1];
                    const int y0 = S.rect[p][2], y1 = S.rect[p][3];
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
            __syncthreads();
        }
        if (S.done) break;
        __syncthreads();
    }

    // ---- write the tile and its FP64 partial totals ----
    const size_t nmesh = (size_t)nc * nc * nc;
    double sn = 0.0, sh = 0.0;
    for (int e = tid; e < TS * TS * TS; e += DEP_THREADS) {
        const int lz = e / (TS * TS), c = e % (TS * TS);
        const int lx = c % TS, ly = c / TS;
        if (lx >= E[0] || ly >= E[1] || lz >= E[2]) continue;
        const float4 A = S.accA[lz][c];
        const float4 B = S.accB[lz][c];
        const float hl = S.accC[lz][c];
        const size_t idx = ((size_t)(O[2] + lz) * nc + (O[1] + ly)) * nc + (O[0] + lx);
        sn += (double)A.x + (double)A.y;
        sh += (double)B.w + (double)hl;
        if (P.density_only) {
            J.mesh[idx] = __fadd_rn(A.x, A.y);
        } else {
            J.mesh[idx] = __fadd_rn(A.x, A.y);
            J.mesh[nmesh + idx] = __fadd_rn(B.w, hl);
            J.mesh[2 * nmesh + idx] = __fadd_rn(A.z, A.w);
            J.mesh[3 * nmesh + 3 * idx] = B.x;
            J.mesh[3 * nmesh + 3 * idx + 1] = B.y;
            J.mesh[3 * nmesh + 3 * idx + 2] = B.z;
        }
    }
    // fixed-order reduction: warp shuffles, then warps in order
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
        J.partial[2 * local] = a;
        J.partial[2 * local + 1] = b;
    }
}

void launch_deposit(const float4* pos, const float4* vel, const int* igrp, const float* rk,
                    const TreeView& t, const DepositParams& p, int total_tiles, int* err,
                    cudaStream_t s)
{
    if (total_tiles <= 0 || t.n <= 0) return;
    const size_t smem = sizeof(DepShared);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    k_deposit<<<total_tiles, DEP_THREADS, smem, s>>>(pos, vel, igrp, rk, t, p, err);
    count_launches(1);
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
