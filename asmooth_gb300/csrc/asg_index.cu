// asg_index.cu -- the spatial index that replaces KDTreeSimple
// (kdtree_balanced.cpp:212-296): particles are put in 48-bit Hilbert order
// (16 bits per axis; Morton order with ASG_SPACE_CURVE=morton) by a stable LSD
// radix sort (each 8-bit digit pass is a counting sort: per-tile
// digit histograms built with warp-aggregated shared-memory atomics, one
// exclusive scan, a stable scatter), then a radix tree (Karras 2012) is built
// over the sorted keys with AABBs computed bottom-up.
//
// Determinism: the sort is stable and starts from input order, so equal keys
// stay in input-index order; the tree is a pure function of the sorted keys.
#include <atomic>
#include <cstdlib>
#include <cstring>

#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

// ---------------------------------------------------------------------------
// unpack + space-filling-curve keys
// ---------------------------------------------------------------------------
struct ParticleRec {  // struct Particle (basic_types.h:10-15), 36 bytes
    float x[3], v[3];
    float dens, rk;
    int igrp;
};
static_assert(sizeof(ParticleRec) == 36, "Particle record must be 36 bytes");

__global__ void k_unpack_aos(const ParticleRec* __restrict__ aos, int n, float4* __restrict__ pos,
                             float4* __restrict__ vel, int* __restrict__ igrp,
                             float* __restrict__ rkin, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = reinterpret_cast<const float*>(aos + i);
    const float x = r[0], y = r[1], z = r[2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicOr(err, ERR_NONFINITE);
    pos[i] = make_float4(x, y, z, __int_as_float(i));
    vel[i] = make_float4(r[3], r[4], r[5], r[6]);
    igrp[i] = reinterpret_cast<const int*>(r)[8];
    rkin[i] = r[7];
}

__global__ void k_unpack_soa(const float* __restrict__ x3, const float* __restrict__ v3,
                             const float* __restrict__ dens, const int* __restrict__ ig, int n,
                             float4* __restrict__ pos, float4* __restrict__ vel,
                             int* __restrict__ igrp, float* __restrict__ rkin, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = x3[3 * (size_t)i], y = x3[3 * (size_t)i + 1], z = x3[3 * (size_t)i + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicOr(err, ERR_NONFINITE);
    pos[i] = make_float4(x, y, z, __int_as_float(i));
    const float d = dens ? dens[i] : 0.0f;
    vel[i] = v3 ? make_float4(v3[3 * (size_t)i], v3[3 * (size_t)i + 1], v3[3 * (size_t)i + 2], d)
                : make_float4(0.f, 0.f, 0.f, d);
    igrp[i] = ig ? ig[i] : 0;
    rkin[i] = 0.0f;
}

// Mixed-precision input: one int32 cell index c = (cz * grid + cy) * grid + cx
// and three uint16 offsets per particle.  Each coordinate decodes as
//   x = (left + cs * cx) + off * unit,   unit = cs / 65536,
// every product and sum rounded to nearest in this order (the host decode in
// the Python package does the same float32 operations).
__global__ void k_unpack_quant(const int* __restrict__ cell, const uint16_t* __restrict__ off,
                               const float* __restrict__ v3, int n, int grid, float left, float cs,
                               float unit, float4* __restrict__ pos, float4* __restrict__ vel,
                               int* __restrict__ igrp, float* __restrict__ rkin, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell[i];
    const int g2 = grid * grid;
    if (c < 0 || (long long)c >= (long long)g2 * grid) {
        atomicOr(err, ERR_BADCELL);
        c = 0;
    }
    const int cx = c % grid, cy = (c / grid) % grid, cz = c / g2;
    const float x = __fadd_rn(__fadd_rn(left, __fmul_rn(cs, (float)cx)),
                              __fmul_rn((float)off[3 * (size_t)i], unit));
    const float y = __fadd_rn(__fadd_rn(left, __fmul_rn(cs, (float)cy)),
                              __fmul_rn((float)off[3 * (size_t)i + 1], unit));
    const float z = __fadd_rn(__fadd_rn(left, __fmul_rn(cs, (float)cz)),
                              __fmul_rn((float)off[3 * (size_t)i + 2], unit));
    pos[i] = make_float4(x, y, z, __int_as_float(i));
    vel[i] = v3 ? make_float4(v3[3 * (size_t)i], v3[3 * (size_t)i + 1], v3[3 * (size_t)i + 2], 0.0f)
                : make_float4(0.f, 0.f, 0.f, 0.f);
    igrp[i] = 0;
    rkin[i] = 0.0f;
}

void launch_unpack_quant(const int* cell, const uint16_t* off, const float* v, int n, int grid,
                         float left, float cs, float4* pos_in, float4* vel_in, int* igrp_in,
                         float* rk_in, int* err, cudaStream_t s)
{
    if (n <= 0) return;
    const float unit = cs / 65536.0f;
    k_unpack_quant<<<(n + 255) / 256, 256, 0, s>>>(cell, off, v, n, grid, left, cs, unit, pos_in,
                                                    vel_in, igrp_in, rk_in, err);
    count_launches(1);
}

void launch_unpack_aos(const void* aos, int n, float4* pos_in, float4* vel_in, int* igrp_in,
                       float* rk_in, int* err, cudaStream_t s)
{
    if (n <= 0) return;
    k_unpack_aos<<<(n + 255) / 256, 256, 0, s>>>((const ParticleRec*)aos, n, pos_in, vel_in,
                                                  igrp_in, rk_in, err);
    count_launches(1);
}

void launch_unpack_soa(const float* x, const float* v, const float* dens, const int* igrp, int n,
                       float4* pos_in, float4* vel_in, int* igrp_in, float* rk_in, int* err,
                       cudaStream_t s)
{
    if (n <= 0) return;
    k_unpack_soa<<<(n + 255) / 256, 256, 0, s>>>(x, v, dens, igrp, n, pos_in, vel_in, igrp_in,
                                                  rk_in, err);
    count_launches(1);
}

// order-preserving float <-> int map for atomicMin/atomicMax on floats
__device__ __forceinline__ int fkey(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fkey_inv(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void k_bounds_init(int* lohi)
{
    lohi[0] = 0x7fffffff;
    lohi[1] = (int)0x80000000;
}

__global__ void k_bounds(const float4* __restrict__ pos, int n, int* lohi)
{
    float lo = INFINITY, hi = -INFINITY;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        lo = fminf(lo, fminf(p.x, fminf(p.y, p.z)));
        hi = fmaxf(hi, fmaxf(p.x, fmaxf(p.y, p.z)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_down_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_down_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(lohi, fkey(lo));
        atomicMax(lohi + 1, fkey(hi));
    }
}

// space-filling-curve key of each particle: 16 bits per axis over [left,
// right), with the bounds either given (lohi == nullptr) or read from
// k_bounds' output; Hilbert order, or Morton order with hilbert == 0
__global__ void k_space_keys(const float4* __restrict__ pos, int n, float left, float right,
                             const int* __restrict__ lohi, uint64_t prefix, int hilbert,
                             uint64_t* __restrict__ keys, int* __restrict__ vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (lohi) {
        left = fkey_inv(lohi[0]);
        right = fkey_inv(lohi[1]);
    }
    const float w = right - left;
    const float scale = w > 0.0f ? 65536.0f / w : 1.0f;
    const float4 p = pos[i];
    auto cell = [&](float c) -> uint32_t {
        float t = (c - left) * scale;
        t = fminf(fmaxf(t, 0.0f), 65535.0f);
        return (uint32_t)t;
    };
    const uint32_t cx = cell(p.x), cy = cell(p.y), cz = cell(p.z);
    const uint64_t k = hilbert ? hilbert_key48(cx, cy, cz)
                               : spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2);
    keys[i] = (prefix << 48) | k;
    vals[i] = i;
}

// ASG_SPACE_CURVE=morton selects Morton order (a tuning and comparison knob)
static int use_hilbert()
{
    static const int h = [] {
        const char* e = std::getenv("ASG_SPACE_CURVE");
        return (e && std::strcmp(e, "morton") == 0) ? 0 : 1;
    }();
    return h;
}

void launch_space_keys(const float4* pos_in, int n, float left, float right, int* d_lohi,
                       uint64_t key_prefix, uint64_t* keys, int* vals, cudaStream_t s)
{
    if (n <= 0) return;
    if (d_lohi) {
        k_bounds_init<<<1, 1, 0, s>>>(d_lohi);
        k_bounds<<<min((n + 255) / 256, 1216), 256, 0, s>>>(pos_in, n, d_lohi);
        count_launches(2);
    }
    k_space_keys<<<(n + 255) / 256, 256, 0, s>>>(pos_in, n, left, right, d_lohi, key_prefix,
                                                  use_hilbert(), keys, vals);
    count_launches(1);
}

// ---------------------------------------------------------------------------
// exclusive scan (uint32)
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(uint32_t* data, size_t n, uint32_t* sums)
{
    __shared__ uint32_t warp_tot[32];
    const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tot[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warp_tot[lane] = wi - w;  // exclusive warp offsets
        if (lane == 31 && sums) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + inc - t;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_add(uint32_t* data, size_t n, const uint32_t* offs)
{
    const uint32_t o = offs[blockIdx.x];
    const size_t base = (size_t)blockIdx.x * SCAN_TILE;
    for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS)
        if (base + k < n) data[base + k] += o;
}

size_t scan_temp_bytes(size_t n)
{
    size_t total = 0;
    while (n > 1) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        total += n;
    }
    return (total + 64) * sizeof(uint32_t);
}

void exclusive_scan_u32(uint32_t* data, size_t n, void* temp, cudaStream_t s)
{
    if (n == 0) return;
    const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    uint32_t* sums = (uint32_t*)temp;
    k_scan_tiles<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(data, n, nb > 1 ? sums : nullptr);
    count_launches(1);
    if (nb > 1) {
        exclusive_scan_u32(sums, nb, sums + nb, s);
        k_scan_add<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(data, n, sums);
        count_launches(1);
    }
}

// ---------------------------------------------------------------------------
// stable LSD radix sort, 8-bit digits
// ---------------------------------------------------------------------------
#ifndef ASG_RS_ROUNDS
#define ASG_RS_ROUNDS 8
#endif
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = ASG_RS_ROUNDS;  // elements per thread of a tile
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

template <class K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_count(const K* __restrict__ keys, int n,
                                                         int shift, uint32_t* __restrict__ counts,
                                                         int ntiles)
{
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
    const unsigned lane = threadIdx.x & 31;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = base + r * RS_THREADS + threadIdx.x;
        const bool valid = i < n;
        const unsigned d = valid ? (unsigned)((keys[i] >> shift) & 255u) : 256u;
        // warp-aggregated atomics: one shared-memory add per distinct digit
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (valid && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&hist[d], __popc(peers));
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

// Stable scatter of one 8-bit digit.  A block takes a tile of RS_TILE elements;
// warp w ranks its own contiguous RS_ROUNDS x 32 elements with per-warp digit
// counters (no block barrier while ranking), one block-level scan turns the
// counters into positions of the tile in digit order, the tile is placed in
// shared memory in that order, and written out so that consecutive threads
// store consecutive addresses within each digit's run.  Order is kept: within
// a digit, elements stay in (warp, round, lane) = input order.
template <class K>
struct RsScatterSmem {
    K key[RS_TILE];
    int val[RS_TILE];
    uint32_t wcnt[RS_THREADS / 32][256];  // per-warp digit counts, then offsets
    uint32_t lstart[256];                 // first slot of each digit in the tile
    uint32_t gstart[256];                 // the digit's first output position for this tile
};

template <class K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const K* __restrict__ kin,
                                                           const int* __restrict__ vin,
                                                           K* __restrict__ kout,
                                                           int* __restrict__ vout, int n,
                                                           int shift,
                                                           const uint32_t* __restrict__ offs,
                                                           int ntiles)
{
    extern __shared__ __align__(16) unsigned char rs_smem[];
    RsScatterSmem<K>& S = *reinterpret_cast<RsScatterSmem<K>*>(rs_smem);
    const int tid = threadIdx.x, warp = tid >> 5;
    const unsigned lane = tid & 31, lt = lanemask_lt();
    const int base = blockIdx.x * RS_TILE;
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; ++w) S.wcnt[w][tid] = 0u;
    S.gstart[tid] = offs[(size_t)tid * ntiles + blockIdx.x];
    __syncthreads();
    // ---- rank: this warp's elements base + warp*32*ROUNDS + r*32 + lane ----
    K k[RS_ROUNDS];
    int v[RS_ROUNDS];
    uint32_t pos[RS_ROUNDS];  // position among this warp's elements of the same digit
    const int wbase = base + warp * 32 * RS_ROUNDS;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = wbase + r * 32 + (int)lane;
        const bool valid = i < n;
        k[r] = valid ? kin[i] : (K)0;
        v[r] = valid ? vin[i] : 0;
        const unsigned d = valid ? (unsigned)((k[r] >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = valid ? S.wcnt[warp][d] : 0u;
        pos[r] = before + __popc(peers & lt);
        __syncwarp();
        if (valid && (peers & lt) == 0u) S.wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // ---- per digit (thread = digit): offsets of the warps, then the tile's scan ----
    {
        uint32_t sum = 0;
#pragma unroll
        for (int w = 0; w < RS_THREADS / 32; ++w) {
            const uint32_t c = S.wcnt[w][tid];
            S.wcnt[w][tid] = sum;
            sum += c;
        }
        // exclusive scan of the 256 digit totals (one per thread)
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if ((int)lane >= o) inc += y;
        }
        __shared__ uint32_t wsum[RS_THREADS / 32];
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t woff = 0;
        for (int w = 0; w < warp; ++w) woff += wsum[w];
        S.lstart[tid] = woff + inc - sum;
    }
    __syncthreads();
    // ---- place the tile in digit order ----
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int i = wbase + r * 32 + (int)lane;
        if (i < n) {
            const unsigned d = (unsigned)((k[r] >> shift) & 255u);
            const uint32_t slot = S.lstart[d] + S.wcnt[warp][d] + pos[r];
            S.key[slot] = k[r];
            S.val[slot] = v[r];
        }
    }
    __syncthreads();
    // ---- write out: slot j of digit d goes to gstart[d] + (j - lstart[d]) ----
    const int cnt = min(RS_TILE, n - base);
    for (int j = tid; j < cnt; j += RS_THREADS) {
        const K kk = S.key[j];
        const unsigned d = (unsigned)((kk >> shift) & 255u);
        const uint32_t dst = S.gstart[d] + ((uint32_t)j - S.lstart[d]);
        kout[dst] = kk;
        vout[dst] = S.val[j];
    }
}

size_t radix_sort_temp_bytes(int n)
{
    const size_t ntiles = (size_t)(n + RS_TILE - 1) / RS_TILE;
    const size_t nc = 256 * ntiles;
    return nc * sizeof(uint32_t) + scan_temp_bytes(nc) + 256;
}

template <class K>
static int radix_sort_t(K* keys0, int* vals0, K* keys1, int* vals1, int n, int bits, void* temp,
                        cudaStream_t s)
{
    if (n <= 1) return 0;
    const int ntiles = (n + RS_TILE - 1) / RS_TILE;
    static std::atomic<unsigned long long> attr_set{0};  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (!(attr_set.load() & (1ull << (dev & 63)))) {
        cudaFuncSetAttribute(k_rs_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(RsScatterSmem<K>));
        attr_set.fetch_or(1ull << (dev & 63));
    }
    uint32_t* counts = (uint32_t*)temp;
    void* stemp = (void*)(counts + (size_t)256 * ntiles);
    K* kb[2] = {keys0, keys1};
    int* vb[2] = {vals0, vals1};
    int cur = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_count<K><<<ntiles, RS_THREADS, 0, s>>>(kb[cur], n, shift, counts, ntiles);
        exclusive_scan_u32(counts, (size_t)256 * ntiles, stemp, s);
        k_rs_scatter<K><<<ntiles, RS_THREADS, sizeof(RsScatterSmem<K>), s>>>(
            kb[cur], vb[cur], kb[cur ^ 1], vb[cur ^ 1], n, shift, counts, ntiles);
        count_launches(2);
        cur ^= 1;
    }
    return cur;
}

int radix_sort(uint64_t* keys0, int* vals0, uint64_t* keys1, int* vals1, int n, int bits,
               void* temp, cudaStream_t s)
{
    return radix_sort_t<uint64_t>(keys0, vals0, keys1, vals1, n, bits, temp, s);
}

int radix_sort32(uint32_t* keys0, int* vals0, uint32_t* keys1, int* vals1, int n, int bits,
                 void* temp, cudaStream_t s)
{
    return radix_sort_t<uint32_t>(keys0, vals0, keys1, vals1, n, bits, temp, s);
}

__global__ void k_gather(const int* __restrict__ perm, const float4* __restrict__ pos_in,
                         const float4* __restrict__ vel_in, const int* __restrict__ igrp_in,
                         const float* __restrict__ rk_in, int n, float4* __restrict__ pos,
                         float4* __restrict__ vel, int* __restrict__ igrp, float* __restrict__ rk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm[i];
    pos[i] = pos_in[o];
    vel[i] = vel_in[o];
    igrp[i] = igrp_in[o];
    rk[i] = rk_in[o];
}

void launch_gather_sorted(const int* perm, const float4* pos_in, const float4* vel_in,
                          const int* igrp_in, const float* rk_in, int n, float4* pos, float4* vel,
                          int* igrp, float* rk, cudaStream_t s)
{
    if (n <= 0) return;
    k_gather<<<(n + 255) / 256, 256, 0, s>>>(perm, pos_in, vel_in, igrp_in, rk_in, n, pos, vel,
                                              igrp, rk);
    count_launches(1);
}

__global__ void k_iota(int* a, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}
void launch_iota(int* a, int n, cudaStream_t s)
{
    if (n <= 0) return;
    k_iota<<<(n + 255) / 256, 256, 0, s>>>(a, n);
    count_launches(1);
}

__global__ void k_check_rk(const float* __restrict__ rk, int n, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float h = rk[i];
    if (!(h > 0.0f && h < INFINITY)) atomicOr(err, ERR_ZERO_RK);
}
void launch_check_rk(const float* rk, int n, int* err, cudaStream_t s)
{
    if (n <= 0) return;
    k_check_rk<<<(n + 255) / 256, 256, 0, s>>>(rk, n, err);
    count_launches(1);
}

// ---------------------------------------------------------------------------
// radix tree (Karras 2012, "Maximizing parallelism in the construction of
// BVHs, octrees, and k-d trees"); duplicate keys are split by position
// ---------------------------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint64_t* __restrict__ k, int n, int i, long long j)
{
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[(int)j];
    if (a == b) return 64 + __clz(i ^ (int)j);
    return __clzll(a ^ b);
}

__global__ void k_build_tree(const uint64_t* __restrict__ keys, int n, int4* __restrict__ meta,
                             int* __restrict__ parent, int* __restrict__ leaf_parent)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (kdelta(keys, n, i, (long long)i + 1) - kdelta(keys, n, i, (long long)i - 1)) > 0 ? 1 : -1;
    const int dmin = kdelta(keys, n, i, (long long)i - d);
    long long lmax = 2;
    while (kdelta(keys, n, i, (long long)i + lmax * d) > dmin) lmax <<= 1;
    long long l = 0;
    for (long long t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(keys, n, i, (long long)i + (l + t) * d) > dmin) l += t;
    const long long j = (long long)i + l * d;
    const int dnode = kdelta(keys, n, i, j);
    long long s = 0;
    long long t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(keys, n, i, (long long)i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = (int)((long long)i + s * d + (d < 0 ? d : 0));
    const int lo = (int)(i < j ? i : j), hi = (int)(i < j ? j : i);
    const int c0 = (lo == gamma) ? ~gamma : gamma;
    const int c1 = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    meta[i] = make_int4(c0, c1, lo, hi);
    if (c0 < 0) leaf_parent[~c0] = i; else parent[c0] = i;
    if (c1 < 0) leaf_parent[~c1] = i; else parent[c1] = i;
    if (i == 0) parent[0] = -1;
}

void launch_build_tree(const uint64_t* keys, int n, int4* meta, int* parent, int* leaf_parent,
                       cudaStream_t s)
{
    if (n <= 1) {
        if (n == 1) cudaMemsetAsync(leaf_parent, 0xff, sizeof(int), s);
        return;
    }
    k_build_tree<<<(n - 1 + 255) / 256, 256, 0, s>>>(keys, n, meta, parent, leaf_parent);
    count_launches(1);
}

// leaf box: the point itself, or [x-h', x+h'] with h' = rk*(1+1e-6) rounded up and
// the bounds rounded outwards, so that a point outside it is farther than rk
__device__ __forceinline__ void leaf_box(const float4* pos, const float* rk, int i, float4& lo,
                                         float4& hi)
{
    const float4 p = pos[i];
    if (rk) {
        const float h = __fmul_ru(rk[i], 1.000001f);
        lo = make_float4(__fsub_rd(p.x, h), __fsub_rd(p.y, h), __fsub_rd(p.z, h), 0.f);
        hi = make_float4(__fadd_ru(p.x, h), __fadd_ru(p.y, h), __fadd_ru(p.z, h), 0.f);
    } else {
        lo = make_float4(p.x, p.y, p.z, 0.f);
        hi = lo;
    }
}

__device__ __forceinline__ void box_union(float4& l, float4& h, const float4& l1, const float4& h1)
{
    l = make_float4(fminf(l.x, l1.x), fminf(l.y, l1.y), fminf(l.z, l1.z), 0.f);
    h = make_float4(fmaxf(h.x, h1.x), fmaxf(h.y, h1.y), fmaxf(h.z, h1.z), 0.f);
}

// the 64-byte record of node i (TreeView::rec): meta, then the boxes of both
// children as coordinate pairs, or (bucket) the node's own box
__device__ __forceinline__ void write_node_rec(float4* rec, int i, int4 m, float4 l0, float4 h0,
                                               float4 l1, float4 h1)
{
    float4* r = rec + 4 * (size_t)i;
    r[0] = make_float4(__int_as_float(m.x), __int_as_float(m.y), __int_as_float(m.z),
                       __int_as_float(m.w));
    r[1] = make_float4(l0.x, l1.x, l0.y, l1.y);
    r[2] = make_float4(l0.z, l1.z, h0.x, h1.x);
    r[3] = make_float4(h0.y, h1.y, h0.z, h1.z);
}
__device__ __forceinline__ void write_bucket_rec(float4* rec, int i, int4 m, float4 l, float4 h)
{
    float4* r = rec + 4 * (size_t)i;
    r[0] = make_float4(__int_as_float(m.x), __int_as_float(m.y), __int_as_float(m.z),
                       __int_as_float(m.w));
    r[1] = make_float4(l.x, l.y, l.z, h.x);
    r[2] = make_float4(h.y, h.z, 0.f, 0.f);
    r[3] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Boxes of the nodes a traversal can read: the root and every child of a node
// with more than `leaf` particles (the traversals scan smaller nodes whole and
// never look below them).  A "top bucket" (<= leaf particles, parent larger)
// reduces its contiguous particles directly, then climbs: a node with two
// internal children is finished by the second arrival (atomic flag), a node
// with one internal child by its only climber.  Unions of the same particle
// boxes, so the boxes are the same bits as a climb from every particle.  With
// rec, each finished node also gets its record (TreeView::rec): a top bucket
// its own box, a larger node the boxes of its children, which its finisher
// holds at that moment; a node inside a bucket is never visited and gets none.
__global__ void k_tree_boxes(const float4* __restrict__ pos, const float* __restrict__ rk, int n,
                             int leaf, const int4* __restrict__ meta, const int* __restrict__ parent,
                             int* flags, float4* lo, float4* hi, float4* __restrict__ rec)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = i < n - 1;
    const int4 m = valid ? meta[i] : make_int4(0, 0, 0, 0);
    float4 l, h, l1, h1;
    bool start = false;  // this thread finishes node i and climbs from it
    bool top = false;    // node i is a top bucket
    if (valid) {
        if (m.w - m.z + 1 > leaf) {
            start = m.x < 0 && m.y < 0;  // two particle children (leaf = 1 only)
            if (start) {
                leaf_box(pos, rk, ~m.x, l, h);
                leaf_box(pos, rk, ~m.y, l1, h1);
                if (rec) write_node_rec(rec, i, m, l, h, l1, h1);
                box_union(l, h, l1, h1);
            }
        } else {
            const int p = parent[i];
            top = p < 0 || meta[p].w - meta[p].z + 1 > leaf;  // not inside a larger bucket
            start = top;
        }
    }
    // the warp reduces its top buckets one after another, lanes over the
    // bucket's (at most 32) contiguous particles: one coalesced load each
    unsigned tops = __ballot_sync(0xffffffffu, top);
    while (tops) {
        const int src = __ffs(tops) - 1;
        tops &= tops - 1;
        const int first = __shfl_sync(0xffffffffu, m.z, src);
        const int last = __shfl_sync(0xffffffffu, m.w, src);
        float4 bl, bh;
        leaf_box(pos, rk, min(first + lane, last), bl, bh);
        float r[6] = {bl.x, bl.y, bl.z, bh.x, bh.y, bh.z};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                const float v = __shfl_xor_sync(0xffffffffu, r[a], o);
                r[a] = a < 3 ? fminf(r[a], v) : fmaxf(r[a], v);
            }
        if (lane == src) {
            l = make_float4(r[0], r[1], r[2], 0.f);
            h = make_float4(r[3], r[4], r[5], 0.f);
        }
    }
    if (!start) return;
    if (top && rec) write_bucket_rec(rec, i, m, l, h);
    __stcg(&lo[i], l);
    __stcg(&hi[i], h);
    int node = parent[i];
    while (node >= 0) {
        const int4 mm = meta[node];
        if (mm.x >= 0 && mm.y >= 0) {
            __threadfence();
            if (atomicAdd(&flags[node], 1) == 0) return;  // the sibling finishes this node
            __threadfence();
        }
        if (mm.x < 0) leaf_box(pos, rk, ~mm.x, l, h);
        else { l = __ldcg(&lo[mm.x]); h = __ldcg(&hi[mm.x]); }
        if (mm.y < 0) leaf_box(pos, rk, ~mm.y, l1, h1);
        else { l1 = __ldcg(&lo[mm.y]); h1 = __ldcg(&hi[mm.y]); }
        if (rec) write_node_rec(rec, node, mm, l, h, l1, h1);
        box_union(l, h, l1, h1);
        __stcg(&lo[node], l);
        __stcg(&hi[node], h);
        node = parent[node];
    }
}

void launch_tree_boxes(const float4* pos, const float* rk, int n, int leaf, const int4* meta,
                       const int* parent, int* flags, float4* lo, float4* hi, float4* rec,
                       cudaStream_t s)
{
    if (n <= 1) return;
    cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)(n - 1), s);
    k_tree_boxes<<<(n - 1 + 255) / 256, 256, 0, s>>>(pos, rk, n, leaf, meta, parent, flags, lo, hi,
                                                      rec);
    count_launches(1);
}

// ---------------------------------------------------------------------------
// output in input order
// ---------------------------------------------------------------------------
__global__ void k_pack_aos(const int* __restrict__ perm, const float4* __restrict__ pos,
                           const float4* __restrict__ vel, const float* __restrict__ rk,
                           const float* __restrict__ dens, const int* __restrict__ igrp, int n,
                           ParticleRec* __restrict__ aos)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm ? perm[i] : i;  // no perm: the arrays are in output order
    const float4 p = pos[i], v = vel[i];
    float* r = reinterpret_cast<float*>(aos + o);
    r[0] = p.x; r[1] = p.y; r[2] = p.z;
    r[3] = v.x; r[4] = v.y; r[5] = v.z;
    r[6] = dens ? dens[i] : v.w;
    r[7] = rk ? rk[i] : 0.0f;
    reinterpret_cast<int*>(r)[8] = igrp[i];
}

void launch_pack_aos(const int* perm, const float4* pos, const float4* vel, const float* rk,
                     const float* dens, const int* igrp, int n, void* aos, cudaStream_t s)
{
    if (n <= 0) return;
    k_pack_aos<<<(n + 255) / 256, 256, 0, s>>>(perm, pos, vel, rk, dens, igrp, n,
                                                (ParticleRec*)aos);
    count_launches(1);
}

__global__ void k_scatter_fields(const int* __restrict__ perm, const float* __restrict__ rk,
                                 const float* __restrict__ dens, const int* __restrict__ igrp,
                                 int n, float* rk_out, float* dens_out, int* igrp_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm[i];
    if (rk_out) rk_out[o] = rk[i];
    if (dens_out) dens_out[o] = dens[i];
    if (igrp_out) igrp_out[o] = igrp[i];
}

void launch_scatter_fields(const int* perm, const float* rk, const float* dens, const int* igrp,
                           int n, float* rk_out, float* dens_out, int* igrp_out, cudaStream_t s)
{
    if (n <= 0) return;
    k_scatter_fields<<<(n + 255) / 256, 256, 0, s>>>(perm, rk, dens, igrp, n, rk_out, dens_out,
                                                      igrp_out);
    count_launches(1);
}

}  // namespace asg
