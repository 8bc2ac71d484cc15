// asg_noalloc.cu -- a neighbour search that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application that reserves the
// whole GPU memory pool up front for its own allocator and hands libraries
// only the buffers it owns, or code that runs where a device allocation
// (which can synchronise the device) is not allowed.  For them this file
// provides asg_neighbor_search_noalloc: the same kernels as
// asg_neighbor_search, with every scratch array placed in one file-scope
// __device__ array compiled into the library, so the call makes no
// cudaMalloc, cudaFree or other allocating call.  The caller passes its own
// device buffers for the inputs and outputs.
//
// Costs and limits of the fixed scratch:
//   * the array (NOALLOC_BYTES, about 10 MB) takes device memory on a GPU
//     from the moment the library's module is loaded there until the process
//     exits.  With CUDA's lazy module loading (the default) that is the first
//     call into this file on that device, not the dlopen of the library, so a
//     caller that reserves its memory pool up front makes a preparing call
//     (np = 0 and null pointers) on each device before the reservation;
//   * at most NOALLOC_MAX_N particles per call; larger inputs are rejected
//     with ASG_ERR_NOALLOC_LIMIT;
//   * every call on a device uses the same array and leaves the last call's
//     contents in it, so calls that overlap on the GPU (other streams, other
//     host threads) race and must be serialised by the caller;
//   * the first call on each device (the preparing call, or the first search)
//     looks up the array's device address (cudaGetSymbolAddress) and keeps it
//     for later calls; make that first call before any stream capture.  After a
//     cudaDeviceReset the kept address is stale: a preparing call looks it up
//     again;
//   * the call is synchronous: it returns when its work on the stream is done.
#include <mutex>

#include "../../include/asmooth_gb300.h"
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

constexpr int NOALLOC_MAX_N = ASG_NOALLOC_MAX_PARTICLES;
constexpr int NOALLOC_MAX_DEVICES = 64;

// byte offsets of the arrays carved out of the scratch for n particles
struct NoallocLayout {
    size_t pos_in, vel_in, igrp_in, rk_in, keys0, keys1, vals0, vals1, sort_tmp;
    size_t pos, vel, igrp, rk, t33, idx33, meta, parent, leaf_parent, flags;
    size_t blo, bhi, rec, dacc, dexp, err, total;
};

static constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

static NoallocLayout noalloc_layout(size_t n)
{
    NoallocLayout L{};
    const size_t m = n > 1 ? n - 1 : 1;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    L.pos_in = take(16 * n);
    L.vel_in = take(16 * n);
    L.igrp_in = take(4 * n);
    L.rk_in = take(4 * n);
    L.keys0 = take(8 * n);
    L.keys1 = take(8 * n);
    L.vals0 = take(4 * n);
    L.vals1 = take(4 * n);
    L.sort_tmp = take(radix_sort_temp_bytes((int)n));
    L.pos = take(16 * n);
    L.vel = take(16 * n);
    L.igrp = take(4 * n);
    L.rk = take(4 * n);
    L.t33 = take(4 * n);
    L.idx33 = take(4 * n);
    L.meta = take(16 * m);
    L.parent = take(4 * m);
    L.leaf_parent = take(4 * n);
    L.flags = take(4 * m);
    L.blo = take(16 * m);
    L.bhi = take(16 * m);
    L.rec = take(64 * m);
    L.dacc = take(8 * n);
    L.dexp = take(4 * n);
    L.err = take(16);
    L.total = o;
    return L;
}

// 248 bytes per particle in the arrays above plus the radix sort's scratch
// (radix_sort_temp_bytes) and 256-byte alignment of every array: 304 bytes
// per particle and 64 KB cover them (noalloc_layout checks the total)
constexpr size_t NOALLOC_BYTES = 304u * (size_t)NOALLOC_MAX_N + 64u * 1024u;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

static void* g_scratch_ptr[NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mu;

// device address of the scratch on the current device, looked up once per
// device (again when refresh is set: the preparing call)
static int scratch_address(int dev, void** out, bool refresh)
{
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return ASG_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev] || refresh) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return ASG_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return ASG_OK;
}

// sorted rk and dens (vel.w) back to input order, in the caller's buffers
__global__ static void k_noalloc_store(const int* __restrict__ perm, const float* __restrict__ rk,
                                       const float4* __restrict__ vel, int n,
                                       float* __restrict__ rk_out, float* __restrict__ dens_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm[i];
    rk_out[o] = rk[i];
    dens_out[o] = vel[i].w;
}

static int noalloc_status(int bits)
{
    if (bits & ERR_NONFINITE) return ASG_ERR_NONFINITE;
    if (bits & ERR_STACK) return ASG_ERR_STACK;
    if (bits & ERR_FEW) return ASG_ERR_FEW;
    if (bits & ERR_ZERO_RK) return ASG_ERR_ZERO_RK;
    if (bits & ERR_TIES) return ASG_ERR_TIES;
    return ASG_OK;
}

}  // namespace asg

using namespace asg;

extern "C" int asg_neighbor_search_noalloc(const float* d_x, int np, float left, float right,
                                           float* d_rk, float* d_dens, void* stream)
{
    // an unread error of the caller's earlier CUDA work on this thread would be
    // reported as this call's own: refuse before any work and leave it unread
    if (cudaPeekAtLastError() != cudaSuccess) return ASG_ERR_CUDA;
    if (np == 0 && !d_x && !d_rk && !d_dens) {
        // preparing call: load the module on the current device (which places
        // the scratch there) and look up the scratch's address
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) {
            cudaGetLastError();
            return ASG_ERR_CUDA;
        }
        void* base = nullptr;
        return scratch_address(dev, &base, true);
    }
    if (!d_x || !d_rk || !d_dens) return ASG_ERR_ARG;
    if (np < K_NN) return np > 0 ? ASG_ERR_FEW : ASG_ERR_ARG;
    if (np > NOALLOC_MAX_N) return ASG_ERR_NOALLOC_LIMIT;
    if (!(left < right) || !(right - left < INFINITY)) return ASG_ERR_ARG;
    const NoallocLayout L = noalloc_layout((size_t)np);
    if (L.total > NOALLOC_BYTES) return ASG_ERR_NOALLOC_LIMIT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return ASG_ERR_CUDA;
    }
    void* base = nullptr;
    if (int r = scratch_address(dev, &base, false)) return r;
    unsigned char* b = static_cast<unsigned char*>(base);
    auto F4 = [&](size_t off) { return reinterpret_cast<float4*>(b + off); };
    auto F = [&](size_t off) { return reinterpret_cast<float*>(b + off); };
    auto I = [&](size_t off) { return reinterpret_cast<int*>(b + off); };
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int* err = I(L.err);

    // the scratch keeps the previous call's contents: clear the error word
    if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) {
        cudaGetLastError();
        return ASG_ERR_CUDA;
    }
    launch_unpack_soa(d_x, nullptr, d_dens, nullptr, np, F4(L.pos_in), F4(L.vel_in), I(L.igrp_in),
                      F(L.rk_in), err, s);
    launch_space_keys(F4(L.pos_in), np, left, right, nullptr, 0,
                  reinterpret_cast<uint64_t*>(b + L.keys0), I(L.vals0), s);
    const int cur = radix_sort(reinterpret_cast<uint64_t*>(b + L.keys0), I(L.vals0),
                               reinterpret_cast<uint64_t*>(b + L.keys1), I(L.vals1), np, 48,
                               b + L.sort_tmp, s);
    const uint64_t* keys = reinterpret_cast<const uint64_t*>(b + (cur ? L.keys1 : L.keys0));
    const int* perm = I(cur ? L.vals1 : L.vals0);
    launch_gather_sorted(perm, F4(L.pos_in), F4(L.vel_in), I(L.igrp_in), F(L.rk_in), np, F4(L.pos),
                         F4(L.vel), I(L.igrp), F(L.rk), s);
    launch_build_tree(keys, np, reinterpret_cast<int4*>(b + L.meta), I(L.parent), I(L.leaf_parent),
                      s);
    launch_tree_boxes(F4(L.pos), nullptr, np, LEAF_MAX, reinterpret_cast<int4*>(b + L.meta),
                      I(L.parent), I(L.flags), F4(L.blo), F4(L.bhi), F4(L.rec), s);
    TreeView t;
    t.n = np;
    t.leaf = LEAF_MAX;
    t.meta = reinterpret_cast<const int4*>(b + L.meta);
    t.blo = F4(L.blo);
    t.bhi = F4(L.bhi);
    t.rec = F4(L.rec);
    launch_knn_t33(F4(L.pos), t, F(L.t33), F(L.rk), I(L.idx33), nullptr, err, s);
    launch_knn_ties(F4(L.pos), t, F(L.t33), I(L.idx33), 0, err, s);
    launch_check_rk(F(L.rk), np, err, s);
    launch_dens(F4(L.pos), t, F(L.t33), I(L.idx33), nullptr, F(L.rk), I(L.dexp),
                reinterpret_cast<unsigned long long*>(b + L.dacc), F4(L.vel), err, s);
    k_noalloc_store<<<(np + 255) / 256, 256, 0, s>>>(perm, F(L.rk), F4(L.vel), np, d_rk, d_dens);
    count_launches(1);

    int bits = 0;
    cudaError_t e = cudaMemcpyAsync(&bits, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ASG_ERR_CUDA;
    }
    return noalloc_status(bits);
}
