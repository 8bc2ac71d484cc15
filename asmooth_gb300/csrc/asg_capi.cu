// asg_capi.cu -- context, device memory and the C ABI (include/asmooth_gb300.h).
//
// One context owns one CUDA stream and grow-only device buffers sized for the
// largest particle set seen.  Each public call validates its arguments, queues
// its kernels on the context stream, synchronises once at the end and turns
// the device error word into a status code.
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/asmooth_gb300.h"
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {
static std::atomic<long long> g_launches{0};
void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
}  // namespace asg

using namespace asg;

namespace {

struct Buf {
    void* p = nullptr;
    size_t cap = 0;
};

struct MeshBuf {
    Buf mesh, partial;
    int nc = 0;
    size_t words = 0;
};

}  // namespace

struct asg_ctx {
    int device = 0;
    cudaStream_t s = nullptr;
    cudaStream_t s_out = nullptr;      // per-particle outputs copied out while the deposit runs
    cudaEvent_t fields_ready = nullptr;
    int* d_err = nullptr;
    int* h_err = nullptr;  // pinned
    std::string last;

    // loaded particle set
    int n = 0;
    float left = 0.f, right = 0.f;
    bool loaded = false, knn_done = false, rk_checked = false, idx33_all = false;
    int leaf = 32;  // tree bucket size scanned whole by the traversals (fastest on GB300)
    int dep_seg = 4096;  // pairs per deposit work item
    int knn_warps = 2;   // warps per block of the neighbour search (2 or 4)
    int dep_mma = deposit_default_mma();  // deposit engine: tensor cores (1, 2) or CUDA cores (0)
    int* perm = nullptr;       // sorted position -> input index
    uint64_t* keys = nullptr;  // sorted keys

    Buf aos, pos_in, vel_in, igrp_in, rk_in, keys0, keys1, vals0, vals1, sort_tmp;
    Buf pos, vel, igrp, rk, t33, idx33;
    Buf meta, parent, leaf_parent, flags, blo, bhi;
    Buf dacc, dexp;  // dens: fixed-point sums and scale exponents
    Buf blist;       // buckets each bundle's neighbour search scanned
    Buf nrec;        // tree node records (TreeView::rec)
    Buf dep_order;   // the deposit's tile processing order and its inverse
    std::vector<int> dep_order_key;  // the mesh sizes dep_order was made for
    bool dep_order_on = true;        // ASG_DEPOSIT_ORDER=tile: tile order
    Buf uf, minin, mark, scan_tmp, lab_cnt, lab_scan;
    Buf halos, hcount, hmass;
    Buf totals, lohi;
    Buf dep_rec, dep_pcount, dep_tiles, dep_counter, dep_pairs, dep_sort, dep_partial;
    Buf cat, cat_out;  // FOF catalogue scratch and records
    Buf sh_in, sh_all; // periodic shell: interior input + bin sort, all copies + flags
    Buf dec_raw, dec_scan;  // file payloads on the device, zip count scans
    int dec_n = 0;          // particles of the last decode (in sh_in), 0 = none
    uint32_t dep_npairs = 0;
    int dep_tiles_n = 0;
    uint32_t* h_u32 = nullptr;      // pinned, mapped
    uint32_t* h_u32_dev = nullptr;  // its device address
    float mesh_boxsize = 0.0f;
    std::vector<MeshBuf> meshes;

    // phase timing (CUDA events on the context stream)
    bool timing = false;
    double phase_ms[ASG_NPHASES] = {};
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    int open_phase = -1;
    cudaEvent_t open_ev = nullptr;
};

namespace {

int fail(asg_ctx* c, int code, const std::string& msg)
{
    if (c) c->last = msg;
    return code;
}

int cuda_fail(asg_ctx* c, cudaError_t e, const char* where)
{
    return fail(c, ASG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                    \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);    \
    } while (0)

int grow(asg_ctx* ctx, Buf& b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return 0;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    const size_t want = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, ASG_ERR_NOMEM, "cudaMalloc of " + std::to_string(want) + " bytes failed");
    }
    b.cap = want;
    return 0;
}

template <class T>
T* P(Buf& b) { return reinterpret_cast<T*>(b.p); }

int device_status(int bits)
{
    if (bits & ERR_NONFINITE) return ASG_ERR_NONFINITE;
    if (bits & ERR_STACK) return ASG_ERR_STACK;
    if (bits & ERR_FEW) return ASG_ERR_FEW;
    if (bits & ERR_ZERO_RK) return ASG_ERR_ZERO_RK;
    if (bits & ERR_TIES) return ASG_ERR_TIES;
    if (bits & ERR_RANGE) return ASG_ERR_RANGE;
    if (bits & ERR_UF) return ASG_ERR_UNIONFIND;
    if (bits & ERR_BADCELL) return ASG_ERR_ARG;
    if (bits & ERR_CAP) return ASG_ERR_STATE;
    return ASG_OK;
}

cudaEvent_t next_event(asg_ctx* ctx)
{
    if (ctx->ev_used == ctx->ev_pool.size()) {
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        ctx->ev_pool.push_back(e);
    }
    return ctx->ev_pool[ctx->ev_used++];
}

// phase markers: phase_begin(ctx, p) ... phase_end(ctx) bracket queued kernels
void phase_begin(asg_ctx* ctx, int phase)
{
    if (!ctx->timing) return;
    ctx->open_phase = phase;
    ctx->open_ev = next_event(ctx);
    cudaEventRecord(ctx->open_ev, ctx->s);
}

void phase_end(asg_ctx* ctx)
{
    if (!ctx->timing || ctx->open_phase < 0) return;
    cudaEvent_t e = next_event(ctx);
    cudaEventRecord(e, ctx->s);
    ctx->pending.push_back({ctx->open_phase, {ctx->open_ev, e}});
    ctx->open_phase = -1;
}

// Reads one or two device words into ctx->h_u32 and waits for them.  A kernel
// stores them through the mapped host words: a copy would queue on the copy
// engine behind any large device-to-host copy in flight on another stream.
__global__ void k_read_words(const uint32_t* a, const uint32_t* b, uint32_t* out)
{
    out[0] = *a;
    if (b) out[1] = *b;
}

static int read_words(asg_ctx* ctx, const uint32_t* a, const uint32_t* b = nullptr)
{
    k_read_words<<<1, 1, 0, ctx->s>>>(a, b, ctx->h_u32_dev);
    count_launches(1);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->s));
    return 0;
}

// wait for the queued work and report device-side and launch errors
int finish(asg_ctx* ctx, const char* what)
{
    CK(cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    for (auto& pe : ctx->pending) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, pe.second.first, pe.second.second) == cudaSuccess)
            ctx->phase_ms[pe.first] += ms;
    }
    ctx->pending.clear();
    ctx->ev_used = 0;
    ctx->open_phase = -1;
    const int bits = *ctx->h_err;
    if (bits) {
        CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
        return fail(ctx, device_status(bits),
                    std::string(what) + ": device error bits " + std::to_string(bits));
    }
    return ASG_OK;
}

TreeView tree_view(asg_ctx* ctx)
{
    TreeView t;
    t.n = ctx->n;
    t.leaf = ctx->leaf;
    t.meta = P<int4>(ctx->meta);
    t.blo = P<float4>(ctx->blo);
    t.bhi = P<float4>(ctx->bhi);
    t.rec = P<float4>(ctx->nrec);
    return t;
}

int alloc_set(asg_ctx* ctx, int n)
{
    const size_t N = (size_t)n, M = (size_t)(n > 1 ? n - 1 : 1);
    int r = 0;
    r |= grow(ctx, ctx->pos_in, 16 * N);
    r |= grow(ctx, ctx->vel_in, 16 * N);
    r |= grow(ctx, ctx->igrp_in, 4 * N);
    r |= grow(ctx, ctx->rk_in, 4 * N);
    r |= grow(ctx, ctx->keys0, 8 * N);
    r |= grow(ctx, ctx->keys1, 8 * N);
    r |= grow(ctx, ctx->vals0, 4 * N);
    r |= grow(ctx, ctx->vals1, 4 * N);
    r |= grow(ctx, ctx->sort_tmp, radix_sort_temp_bytes(n));
    r |= grow(ctx, ctx->pos, 16 * N);
    r |= grow(ctx, ctx->vel, 16 * N);
    r |= grow(ctx, ctx->igrp, 4 * N);
    r |= grow(ctx, ctx->rk, 4 * N);
    r |= grow(ctx, ctx->t33, 4 * N);
    r |= grow(ctx, ctx->idx33, 4 * N);
    r |= grow(ctx, ctx->meta, 16 * M);
    r |= grow(ctx, ctx->parent, 4 * M);
    r |= grow(ctx, ctx->leaf_parent, 4 * N);
    r |= grow(ctx, ctx->flags, 4 * M);
    r |= grow(ctx, ctx->blo, 16 * M);
    r |= grow(ctx, ctx->bhi, 16 * M);
    r |= grow(ctx, ctx->nrec, 64 * M);
    r |= grow(ctx, ctx->dacc, 8 * N);
    r |= grow(ctx, ctx->dexp, 4 * N);
    r |= grow(ctx, ctx->blist, 4 * knn_list_words(n));
    return r ? ASG_ERR_NOMEM : 0;
}

// sort the staged SoA (pos_in/vel_in/igrp_in/rk_in + keys0/vals0) and build the tree
int build_index(asg_ctx* ctx)
{
    const int n = ctx->n;
    const int cur = radix_sort(P<uint64_t>(ctx->keys0), P<int>(ctx->vals0), P<uint64_t>(ctx->keys1),
                               P<int>(ctx->vals1), n, 48, ctx->sort_tmp.p, ctx->s);
    ctx->keys = cur ? P<uint64_t>(ctx->keys1) : P<uint64_t>(ctx->keys0);
    ctx->perm = cur ? P<int>(ctx->vals1) : P<int>(ctx->vals0);
    launch_gather_sorted(ctx->perm, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                         P<int>(ctx->igrp_in), P<float>(ctx->rk_in), n, P<float4>(ctx->pos),
                         P<float4>(ctx->vel), P<int>(ctx->igrp), P<float>(ctx->rk), ctx->s);
    launch_build_tree(ctx->keys, n, P<int4>(ctx->meta), P<int>(ctx->parent),
                      P<int>(ctx->leaf_parent), ctx->s);
    launch_tree_boxes(P<float4>(ctx->pos), nullptr, n, ctx->leaf, P<int4>(ctx->meta),
                      P<int>(ctx->parent), P<int>(ctx->flags), P<float4>(ctx->blo),
                      P<float4>(ctx->bhi), P<float4>(ctx->nrec), ctx->s);
    phase_end(ctx);
    ctx->loaded = true;
    ctx->knn_done = false;
    ctx->rk_checked = false;
    return 0;
}

int check_bounds(asg_ctx* ctx, int np, float left, float right)
{
    if (np <= 0) return fail(ctx, ASG_ERR_ARG, "np must be positive");
    if (!(left < right) || !std::isfinite(left) || !std::isfinite(right))
        return fail(ctx, ASG_ERR_ARG, "need finite left < right");
    return 0;
}

int check_quant(asg_ctx* ctx, int grid, float cell_size, float left, float right)
{
    if (grid <= 0 || grid > 1290 || !(cell_size > 0.0f) || !std::isfinite(cell_size))
        return fail(ctx, ASG_ERR_ARG, "quantisation grid: need 0 < grid <= 1290, cell_size > 0");
    if (!(left + cell_size * (float)grid >= right))
        return fail(ctx, ASG_ERR_ARG, "quantisation grid does not cover [left, right)");
    return 0;
}

// decode mixed-precision positions already on the device and build the index
void load_quant_device(asg_ctx* ctx, const int* d_cell, const uint16_t* d_off, const float* d_v,
                       int np, float left, float right, float cell_size, int grid)
{
    ctx->n = np;
    ctx->left = left;
    ctx->right = right;
    phase_begin(ctx, ASG_PH_INDEX);
    launch_unpack_quant(d_cell, d_off, d_v, np, grid, left, cell_size, P<float4>(ctx->pos_in),
                        P<float4>(ctx->vel_in), P<int>(ctx->igrp_in), P<float>(ctx->rk_in),
                        ctx->d_err, ctx->s);
    launch_space_keys(P<float4>(ctx->pos_in), np, left, right, nullptr, 0, P<uint64_t>(ctx->keys0),
                  P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
}

// host mixed-precision arrays -> one staging buffer [cell | off (16-B padded) | v]
int stage_quant(asg_ctx* ctx, const int* cell, const uint16_t* off, const float* v, int np,
                const int** d_cell, const uint16_t** d_off, const float** d_v)
{
    const size_t n = (size_t)np;
    const size_t o_off = (4 * n + 15) & ~size_t(15);
    const size_t o_v = (o_off + 6 * n + 15) & ~size_t(15);
    if (int r = grow(ctx, ctx->aos, o_v + (v ? 12 * n : 0))) return r;
    unsigned char* b = P<unsigned char>(ctx->aos);
    CK(cudaMemcpyAsync(b, cell, 4 * n, cudaMemcpyHostToDevice, ctx->s));
    CK(cudaMemcpyAsync(b + o_off, off, 6 * n, cudaMemcpyHostToDevice, ctx->s));
    if (v) CK(cudaMemcpyAsync(b + o_v, v, 12 * n, cudaMemcpyHostToDevice, ctx->s));
    *d_cell = reinterpret_cast<const int*>(b);
    *d_off = reinterpret_cast<const uint16_t*>(b + o_off);
    *d_v = v ? reinterpret_cast<const float*>(b + o_v) : nullptr;
    return 0;
}

// the smoothing lengths are checked once per neighbour search
int ensure_rk_checked(asg_ctx* ctx)
{
    if (ctx->rk_checked) return 0;
    phase_begin(ctx, ASG_PH_CHECK);
    launch_check_rk(P<float>(ctx->rk), ctx->n, ctx->d_err, ctx->s);
    phase_end(ctx);
    ctx->rk_checked = true;
    return 0;
}

}  // namespace

extern "C" {

int asg_abi_version(void) { return ASG_ABI_VERSION; }

}  // extern "C"

// ---- huge-page pinned host blocks ------------------------------------------------
namespace {
std::mutex g_host_mu;
std::unordered_map<void*, std::pair<void*, size_t>> g_host_blocks;  // block -> (mapping, length)

size_t huge_page_bytes()
{
    size_t v = 0;
    if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
        unsigned long long u = 0;
        if (std::fscanf(f, "%llu", &u) == 1) v = (size_t)u;
        std::fclose(f);
    }
    return (v >= (1u << 16) && v <= (1ull << 30) && (v & (v - 1)) == 0) ? v : (2u << 20);
}
}  // namespace

extern "C" {

int asg_host_alloc(size_t bytes, void** out)
{
    if (!out) return ASG_ERR_ARG;
    *out = nullptr;
    if (bytes == 0) return ASG_ERR_ARG;
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    const size_t huge = huge_page_bytes();
    // from half a huge page up, whole huge pages (at most 2x the request):
    // a block's pages must be huge for its copies to keep their rate
    const bool use_huge = bytes >= huge / 2;
    const size_t align = use_huge ? huge : page;
    const size_t len = (bytes + align - 1) / align * align;
    const size_t map_len = use_huge ? len + align : len;
    void* base = mmap(nullptr, map_len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (base == MAP_FAILED) return ASG_ERR_NOMEM;
    char* p = reinterpret_cast<char*>(((uintptr_t)base + align - 1) / align * align);
    if (use_huge) madvise(p, len, MADV_HUGEPAGE);  // advice only: base pages if refused
    std::memset(p, 0, len);  // fault the pages in (as huge pages) before they are pinned
    if (cudaHostRegister(p, len, cudaHostRegisterPortable) != cudaSuccess) {
        cudaGetLastError();
        munmap(base, map_len);
        return ASG_ERR_NOMEM;
    }
    std::lock_guard<std::mutex> g(g_host_mu);
    g_host_blocks[p] = {base, map_len};
    *out = p;
    return ASG_OK;
}

int asg_host_free(void* p)
{
    if (!p) return ASG_OK;
    std::pair<void*, size_t> m;
    {
        std::lock_guard<std::mutex> g(g_host_mu);
        auto it = g_host_blocks.find(p);
        if (it == g_host_blocks.end()) return ASG_ERR_ARG;
        m = it->second;
        g_host_blocks.erase(it);
    }
    cudaHostUnregister(p);
    cudaGetLastError();
    munmap(m.first, m.second);
    return ASG_OK;
}

const char* asg_strerror(int status)
{
    switch (status) {
    case ASG_OK: return "ok";
    case ASG_ERR_ARG: return "bad argument";
    case ASG_ERR_CUDA: return "CUDA error";
    case ASG_ERR_NOMEM: return "device memory allocation failed";
    case ASG_ERR_FEW: return "fewer than 33 particles reachable by a query";
    case ASG_ERR_ZERO_RK: return "smoothing length is zero or not finite";
    case ASG_ERR_NONFINITE: return "non-finite particle position";
    case ASG_ERR_STACK: return "tree traversal stack overflow";
    case ASG_ERR_TIES: return "more than 16 exact ties at the 33rd neighbour";
    case ASG_ERR_RANGE: return "periodic kernel support wider than the mesh";
    case ASG_ERR_STATE: return "call order: a required previous step is missing";
    case ASG_ERR_UNIONFIND: return "union-find retry limit reached";
    case ASG_ERR_NOALLOC_LIMIT: return "input larger than the allocation-free entry point's scratch";
    case ASG_ERR_IO: return "output file could not be opened or written";
    default: return "unknown status";
    }
}

const char* asg_last_error(asg_ctx* ctx) { return ctx ? ctx->last.c_str() : "no context"; }

int asg_create(asg_ctx** out, int device)
{
    if (!out) return ASG_ERR_ARG;
    *out = nullptr;
    asg_ctx* ctx = new asg_ctx();
    ctx->device = device;
    if (const char* e = std::getenv("ASG_LEAF_SIZE")) {  // tuning knob (1..32)
        const int v = std::atoi(e);
        if (v >= 1 && v <= LEAF_MAX) ctx->leaf = v;
    }
    if (const char* e = std::getenv("ASG_DEPOSIT_ORDER")) ctx->dep_order_on = std::strcmp(e, "tile") != 0;
    if (const char* e = std::getenv("ASG_KNN_WARPS")) {  // tuning knob: 2 or 4 warps per block
        const int v = std::atoi(e);
        if (v == 2 || v == 4) ctx->knn_warps = v;
    }
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->s_out, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fields_ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_err, sizeof(int));
    if (e == cudaSuccess) e = cudaHostAlloc(&ctx->h_u32, 4 * sizeof(uint32_t), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(&ctx->h_u32_dev, ctx->h_u32, 0);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        asg_destroy(ctx);
        return ASG_ERR_CUDA;
    }
    *out = ctx;
    return ASG_OK;
}

void asg_destroy(asg_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->s) cudaStreamSynchronize(ctx->s);
    Buf* bufs[] = {&ctx->aos, &ctx->pos_in, &ctx->vel_in, &ctx->igrp_in, &ctx->rk_in,
                   &ctx->keys0, &ctx->keys1, &ctx->vals0, &ctx->vals1, &ctx->sort_tmp,
                   &ctx->pos, &ctx->vel, &ctx->igrp, &ctx->rk, &ctx->t33, &ctx->idx33,
                   &ctx->meta, &ctx->parent, &ctx->leaf_parent, &ctx->flags, &ctx->blo,
                   &ctx->bhi, &ctx->dacc, &ctx->dexp, &ctx->blist, &ctx->nrec, &ctx->dep_order, &ctx->uf, &ctx->minin, &ctx->mark,
                   &ctx->scan_tmp, &ctx->lab_cnt, &ctx->lab_scan, &ctx->halos, &ctx->hcount,
                   &ctx->hmass, &ctx->totals, &ctx->lohi, &ctx->dep_rec, &ctx->dep_pcount,
                   &ctx->dep_tiles, &ctx->dep_counter, &ctx->dep_pairs, &ctx->dep_sort,
                   &ctx->dep_partial, &ctx->cat, &ctx->cat_out, &ctx->sh_in, &ctx->sh_all,
                   &ctx->dec_raw, &ctx->dec_scan};
    for (Buf* b : bufs)
        if (b->p) cudaFree(b->p);
    for (auto& m : ctx->meshes) {
        if (m.mesh.p) cudaFree(m.mesh.p);
        if (m.partial.p) cudaFree(m.partial.p);
    }
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->h_u32) cudaFreeHost(ctx->h_u32);
    if (ctx->s) cudaStreamDestroy(ctx->s);
    if (ctx->s_out) {
        cudaStreamSynchronize(ctx->s_out);
        cudaStreamDestroy(ctx->s_out);
    }
    if (ctx->fields_ready) cudaEventDestroy(ctx->fields_ready);
    delete ctx;
}

void* asg_stream(asg_ctx* ctx) { return ctx ? (void*)ctx->s : nullptr; }
long long asg_kernel_launches(asg_ctx*) { return g_launches.load(); }

// ---- periodic shell of a single-cube run ----------------------------------------------

struct ShellIn {  // interior particles + bin sort scratch inside ctx->sh_in
    size_t pos, vel, igrp, rk, k0, k1, v0, v1, tmp, start, end, total;
};

static ShellIn shell_in_layout(int n)
{
    ShellIn L{};
    const size_t N = (size_t)n;
    size_t o = 0;
    auto take = [&](size_t b) {
        const size_t at = o;
        o = (o + b + 255) & ~size_t(255);
        return at;
    };
    L.pos = take(16 * N);
    L.vel = take(16 * N);
    L.igrp = take(4 * N);
    L.rk = take(4 * N);
    L.k0 = take(4 * N);
    L.k1 = take(4 * N);
    L.v0 = take(4 * N);
    L.v1 = take(4 * N);
    L.tmp = take(radix_sort_temp_bytes(n));
    L.start = take(27 * 4);
    L.end = take(27 * 4);
    L.total = o;
    return L;
}

static int check_shell(asg_ctx* ctx, int np, float boxsize, float bf)
{
    if (np <= 0) return fail(ctx, ASG_ERR_ARG, "np must be positive");
    if (!(boxsize > 0.0f) || !std::isfinite(boxsize) || !(bf > 0.0f) || !(bf < 0.5f))
        return fail(ctx, ASG_ERR_ARG, "need boxsize > 0 and 0 < buffer_factor < 0.5");
    return 0;
}

// sh_in holds the interior particles (unpacked); build the shell and load the set
static int load_shell(asg_ctx* ctx, int np, float boxsize, float bf, int* np_with, int* np_local)
{
    const ShellIn L = shell_in_layout(np);
    unsigned char* b = P<unsigned char>(ctx->sh_in);
    auto F4 = [&](size_t o) { return reinterpret_cast<float4*>(b + o); };
    auto U = [&](size_t o) { return reinterpret_cast<uint32_t*>(b + o); };
    auto I = [&](size_t o) { return reinterpret_cast<int*>(b + o); };
    const float lt = bf * boxsize, rt = (1.0f - bf) * boxsize;  // exchange_buffer.cpp:23-24
    const uint32_t* keys = nullptr;
    const int* order = nullptr;
    launch_shell_bins(F4(L.pos), np, lt, rt, U(L.k0), I(L.v0), U(L.k1), I(L.v1), b + L.tmp,
                      U(L.start), U(L.end), &keys, &order, ctx->s);
    uint32_t se[54];
    CK(cudaMemcpyAsync(se, b + L.start, 27 * 4, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(se + 27, b + L.end, 27 * 4, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    // the reference's send loop order (exchange_buffer.cpp:120-150): source bin, then direction
    ShellPlan plan;
    size_t off = (size_t)np;
    for (int i = 0; i < 27; ++i)
        for (int j = 0; j < 27; ++j) {
            plan.base[i][j] = -1;
            if (i == 13 || j == 13) continue;
            bool send = true;
            for (int a = 0, bi = i, dj = j; a < 3; ++a, bi /= 3, dj /= 3)
                send = send && (dj % 3 == 1 || dj % 3 == bi % 3);
            if (!send) continue;
            plan.base[i][j] = (int)off;
            off += se[27 + i] - se[i];
        }
    if (off > (size_t)INT_MAX) return fail(ctx, ASG_ERR_ARG, "shell too large for int indices");
    const int n_all = (int)off;
    const size_t A = (size_t)n_all;
    const size_t o_vel = 16 * A, o_igrp = 32 * A, o_rk = 36 * A, o_flags = 40 * A;
    const size_t o_scan = (o_flags + 4 * (A + 1) + 255) & ~size_t(255);
    if (int r = grow(ctx, ctx->sh_all, o_scan + scan_temp_bytes(A + 1))) return r;
    if (int r = alloc_set(ctx, n_all)) return r;  // the kept set is at most n_all
    unsigned char* a = P<unsigned char>(ctx->sh_all);
    launch_shell_emit(F4(L.pos), F4(L.vel), I(L.igrp), reinterpret_cast<float*>(b + L.rk), keys,
                      order, U(L.start), np, plan, boxsize, reinterpret_cast<float4*>(a),
                      reinterpret_cast<float4*>(a + o_vel), reinterpret_cast<int*>(a + o_igrp),
                      reinterpret_cast<float*>(a + o_rk), ctx->s);
    const float dx = bf * boxsize;  // clumping_tree_main.cpp:556-558
    uint32_t* flags = reinterpret_cast<uint32_t*>(a + o_flags);
    launch_shell_filter(reinterpret_cast<float4*>(a), reinterpret_cast<float4*>(a + o_vel),
                        reinterpret_cast<int*>(a + o_igrp), reinterpret_cast<float*>(a + o_rk),
                        n_all, -dx, boxsize + dx, flags, a + o_scan, P<float4>(ctx->pos_in),
                        P<float4>(ctx->vel_in), P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->s);
    if (int r = read_words(ctx, flags + n_all, flags + np)) return r;
    const int n = (int)ctx->h_u32[0];
    if (np_with) *np_with = n;
    if (np_local) *np_local = (int)ctx->h_u32[1];
    if (n < K_NN) return fail(ctx, ASG_ERR_FEW, "fewer than 33 particles with the shell");
    ctx->n = n;
    ctx->left = -dx;
    ctx->right = boxsize + dx;
    phase_begin(ctx, ASG_PH_INDEX);
    launch_space_keys(P<float4>(ctx->pos_in), n, ctx->left, ctx->right, nullptr, 0,
                  P<uint64_t>(ctx->keys0), P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
    int r = finish(ctx, "load_periodic_cube");
    if (r) ctx->loaded = false;
    return r;
}

// ---- staged interface ---------------------------------------------------------

int asg_load_particles(asg_ctx* ctx, const asg_particle* p, int np, float left, float right)
{
    if (!ctx || !p) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (int r = check_bounds(ctx, np, left, right)) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    if (int r = grow(ctx, ctx->aos, sizeof(asg_particle) * (size_t)np)) return r;
    ctx->n = np;
    ctx->left = left;
    ctx->right = right;
    phase_begin(ctx, ASG_PH_UPLOAD);
    CK(cudaMemcpyAsync(ctx->aos.p, p, sizeof(asg_particle) * (size_t)np, cudaMemcpyHostToDevice,
                       ctx->s));
    phase_end(ctx);
    phase_begin(ctx, ASG_PH_INDEX);
    launch_unpack_aos(ctx->aos.p, np, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                      P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    launch_space_keys(P<float4>(ctx->pos_in), np, left, right, nullptr, 0, P<uint64_t>(ctx->keys0),
                  P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
    int r = finish(ctx, "load");
    if (r) ctx->loaded = false;
    return r;
}

int asg_load_particles_device(asg_ctx* ctx, const float* d_x, const float* d_v,
                              const float* d_dens, const int* d_igrp, int np, float left,
                              float right)
{
    if (!ctx || !d_x) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (int r = check_bounds(ctx, np, left, right)) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    ctx->n = np;
    ctx->left = left;
    ctx->right = right;
    phase_begin(ctx, ASG_PH_INDEX);
    launch_unpack_soa(d_x, d_v, d_dens, d_igrp, np, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                      P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    launch_space_keys(P<float4>(ctx->pos_in), np, left, right, nullptr, 0, P<uint64_t>(ctx->keys0),
                  P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
    int r = finish(ctx, "load_device");
    if (r) ctx->loaded = false;
    return r;
}

int asg_load_particles_quantised(asg_ctx* ctx, const int* cell, const uint16_t* off,
                                 const float* v, int np, float left, float right, float cell_size,
                                 int grid)
{
    if (!ctx || !cell || !off) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (int r = check_bounds(ctx, np, left, right)) return r;
    if (int r = check_quant(ctx, grid, cell_size, left, right)) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    const int* dc = nullptr;
    const uint16_t* doff = nullptr;
    const float* dv = nullptr;
    if (int r = stage_quant(ctx, cell, off, v, np, &dc, &doff, &dv)) return r;
    load_quant_device(ctx, dc, doff, dv, np, left, right, cell_size, grid);
    int r = finish(ctx, "load_quantised");
    if (r) ctx->loaded = false;
    return r;
}

int asg_load_particles_quantised_device(asg_ctx* ctx, const int* d_cell, const uint16_t* d_off,
                                        const float* d_v, int np, float left, float right,
                                        float cell_size, int grid)
{
    if (!ctx || !d_cell || !d_off) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (int r = check_bounds(ctx, np, left, right)) return r;
    if (int r = check_quant(ctx, grid, cell_size, left, right)) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    load_quant_device(ctx, d_cell, d_off, d_v, np, left, right, cell_size, grid);
    int r = finish(ctx, "load_quantised_device");
    if (r) ctx->loaded = false;
    return r;
}

int asg_load_periodic_cube(asg_ctx* ctx, const asg_particle* p, int np_local, float boxsize,
                           float buffer_factor, int* np_with_buffers, int* np_local_kept)
{
    if (!ctx || !p) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (int r = check_shell(ctx, np_local, boxsize, buffer_factor)) return r;
    CK(cudaSetDevice(ctx->device));
    ctx->loaded = false;
    const ShellIn L = shell_in_layout(np_local);
    if (int r = grow(ctx, ctx->sh_in, L.total)) return r;
    if (int r = grow(ctx, ctx->aos, sizeof(asg_particle) * (size_t)np_local)) return r;
    CK(cudaMemcpyAsync(ctx->aos.p, p, sizeof(asg_particle) * (size_t)np_local,
                       cudaMemcpyHostToDevice, ctx->s));
    unsigned char* b = P<unsigned char>(ctx->sh_in);
    launch_unpack_aos(ctx->aos.p, np_local, reinterpret_cast<float4*>(b + L.pos),
                      reinterpret_cast<float4*>(b + L.vel), reinterpret_cast<int*>(b + L.igrp),
                      reinterpret_cast<float*>(b + L.rk), ctx->d_err, ctx->s);
    ctx->dec_n = np_local;  // sh_in now holds these interior particles
    return load_shell(ctx, np_local, boxsize, buffer_factor, np_with_buffers, np_local_kept);
}

int asg_load_periodic_cube_device(asg_ctx* ctx, const float* d_x, const float* d_v, int np_local,
                                  float boxsize, float buffer_factor, int* np_with_buffers,
                                  int* np_local_kept)
{
    if (!ctx || !d_x) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (int r = check_shell(ctx, np_local, boxsize, buffer_factor)) return r;
    CK(cudaSetDevice(ctx->device));
    ctx->loaded = false;
    const ShellIn L = shell_in_layout(np_local);
    if (int r = grow(ctx, ctx->sh_in, L.total)) return r;
    unsigned char* b = P<unsigned char>(ctx->sh_in);
    launch_unpack_soa(d_x, d_v, nullptr, nullptr, np_local, reinterpret_cast<float4*>(b + L.pos),
                      reinterpret_cast<float4*>(b + L.vel), reinterpret_cast<int*>(b + L.igrp),
                      reinterpret_cast<float*>(b + L.rk), ctx->d_err, ctx->s);
    ctx->dec_n = np_local;  // sh_in now holds these interior particles
    return load_shell(ctx, np_local, boxsize, buffer_factor, np_with_buffers, np_local_kept);
}

// ---- particle files decoded on the device ---------------------------------------------

static size_t a16(size_t v) { return (v + 15) & ~size_t(15); }

int asg_decode_xv(asg_ctx* ctx, const float* xv, int np, const float* shift)
{
    if (!ctx || !xv || !shift || np <= 0) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    ctx->dec_n = 0;
    const ShellIn L = shell_in_layout(np);
    if (int r = grow(ctx, ctx->sh_in, L.total)) return r;
    if (int r = grow(ctx, ctx->dec_raw, 24 * (size_t)np)) return r;
    CK(cudaMemcpyAsync(ctx->dec_raw.p, xv, 24 * (size_t)np, cudaMemcpyHostToDevice, ctx->s));
    unsigned char* b = P<unsigned char>(ctx->sh_in);
    launch_decode_xv(P<float>(ctx->dec_raw), np, shift, reinterpret_cast<float4*>(b + L.pos),
                     reinterpret_cast<float4*>(b + L.vel), reinterpret_cast<int*>(b + L.igrp),
                     reinterpret_cast<float*>(b + L.rk), ctx->d_err, ctx->s);
    if (int r = finish(ctx, "decode_xv")) return r;
    ctx->dec_n = np;
    return ASG_OK;
}

int asg_decode_zip(asg_ctx* ctx, const uint8_t* zip0, const int16_t* zip1, const uint8_t* zip2,
                   const int* zip3, int n_zip3, int np_local, int nc_node_dim, int mesh_scale,
                   float v_r2i, const float* shift)
{
    if (!ctx || !zip2 || !shift || (n_zip3 > 0 && !zip3) || n_zip3 < 0 || np_local < 0 ||
        (np_local > 0 && (!zip0 || !zip1)) || nc_node_dim <= 0 || nc_node_dim > 1290 ||
        mesh_scale <= 0)
        return fail(ctx, ASG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    ctx->dec_n = 0;
    const int nc = nc_node_dim, ncell = nc * nc * nc;
    const size_t N = (size_t)np_local;
    const size_t o3 = a16((size_t)ncell), o0 = o3 + a16(4 * (size_t)n_zip3), o1 = o0 + a16(3 * N);
    if (int r = grow(ctx, ctx->dec_raw, o1 + 6 * N)) return r;
    if (int r = grow(ctx, ctx->dec_scan, zip_scratch_bytes(ncell))) return r;
    const ShellIn L = shell_in_layout(np_local > 0 ? np_local : 1);
    if (int r = grow(ctx, ctx->sh_in, L.total)) return r;
    unsigned char* raw = P<unsigned char>(ctx->dec_raw);
    CK(cudaMemcpyAsync(raw, zip2, (size_t)ncell, cudaMemcpyHostToDevice, ctx->s));
    if (n_zip3) CK(cudaMemcpyAsync(raw + o3, zip3, 4 * (size_t)n_zip3, cudaMemcpyHostToDevice, ctx->s));
    if (N) {
        CK(cudaMemcpyAsync(raw + o0, zip0, 3 * N, cudaMemcpyHostToDevice, ctx->s));
        CK(cudaMemcpyAsync(raw + o1, zip1, 6 * N, cudaMemcpyHostToDevice, ctx->s));
    }
    uint32_t* start = nullptr;
    launch_zip_counts(raw, reinterpret_cast<const int*>(raw + o3), n_zip3, ncell, ctx->dec_scan.p,
                      &start, ctx->d_err, ctx->s);
    CK(cudaMemcpyAsync(ctx->h_u32, start + ncell, 4, cudaMemcpyDeviceToHost, ctx->s));
    if (int r = finish(ctx, "decode_zip counts")) return r;
    if (ctx->h_u32[0] != (uint32_t)np_local)  // file_reader2.cpp:261-264
        return fail(ctx, ASG_ERR_ARG, "zip cell counts sum to " + std::to_string(ctx->h_u32[0]) +
                                          ", the header says " + std::to_string(np_local));
    unsigned char* b = P<unsigned char>(ctx->sh_in);
    launch_zip_particles(raw + o0, reinterpret_cast<const int16_t*>(raw + o1), start, ncell, nc,
                         np_local, mesh_scale, v_r2i, shift, reinterpret_cast<float4*>(b + L.pos),
                         reinterpret_cast<float4*>(b + L.vel), reinterpret_cast<int*>(b + L.igrp),
                         reinterpret_cast<float*>(b + L.rk), ctx->s);
    if (int r = finish(ctx, "decode_zip")) return r;
    ctx->dec_n = np_local;
    return ASG_OK;
}

static bool read_file(const std::string& name, std::vector<unsigned char>& out)
{
    FILE* fp = std::fopen(name.c_str(), "rb");
    if (!fp) return false;
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    out.resize(sz > 0 ? (size_t)sz : 0);
    const bool ok = sz >= 0 && std::fread(out.data(), 1, out.size(), fp) == out.size();
    std::fclose(fp);
    return ok;
}

int asg_read_pm_file_xv(asg_ctx* ctx, const char* filebase, const char* redshift, int inode,
                        const float* shift, int* np)
{
    if (!ctx || !filebase || !redshift || !shift || !np) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    const std::string i = std::to_string(inode);
    const std::string name = std::string(filebase) + i + "/" + redshift + "xv" + i + ".dat";
    std::vector<unsigned char> buf;
    if (!read_file(name, buf)) return fail(ctx, ASG_ERR_IO, "cannot read " + name);
    int n = 0;
    if (buf.size() < 48) return fail(ctx, ASG_ERR_ARG, name + ": short header");
    std::memcpy(&n, buf.data(), 4);  // P3m_header.np_local (file_reader2.cpp:10-14)
    if (n <= 0 || buf.size() < 48 + 24 * (size_t)n)
        return fail(ctx, ASG_ERR_ARG, name + ": np_local does not match the file size");
    *np = n;
    return asg_decode_xv(ctx, reinterpret_cast<const float*>(buf.data() + 48), n, shift);
}

int asg_read_pm_file_zip(asg_ctx* ctx, const char* filebase, const char* redshift, int inode,
                         int nc_node_dim, int mesh_scale, const float* shift, int* np,
                         float* boxsize)
{
    if (!ctx || !filebase || !redshift || !shift || !np || nc_node_dim <= 0 || nc_node_dim > 1290)
        return fail(ctx, ASG_ERR_ARG, "bad arguments");
    const std::string i = std::to_string(inode);
    std::vector<unsigned char> z[4];
    for (int k = 0; k < 4; ++k) {
        const std::string name = std::string(filebase) + i + "/" + redshift + "zip" +
                                 std::to_string(k) + "_" + i + ".dat";
        if (!read_file(name, z[k])) return fail(ctx, ASG_ERR_IO, "cannot read " + name);
    }
    if (z[0].size() < 64 || z[1].size() < 64) return fail(ctx, ASG_ERR_ARG, "short zip header");
    int n = 0;
    float v_r2i = 0.0f;
    std::memcpy(&n, z[0].data(), 4);            // P3m_zip_header0.np_local
    std::memcpy(&v_r2i, z[0].data() + 48, 4);   // P3m_zip_header0.v_r2i (word 12)
    const size_t ncell = (size_t)nc_node_dim * nc_node_dim * nc_node_dim;
    // the reference reads to the exact end of zip0 and zip1 (file_reader2.cpp:254-261)
    if (n < 0 || z[0].size() != 64 + 3 * (size_t)n || z[1].size() != 64 + 6 * (size_t)n ||
        z[2].size() < ncell)
        return fail(ctx, ASG_ERR_ARG, "zip file sizes do not match np_local and nc_node_dim");
    *np = n;
    if (boxsize) *boxsize = (float)(mesh_scale * nc_node_dim);  // file_reader2.cpp:266
    return asg_decode_zip(ctx, z[0].data() + 64, reinterpret_cast<const int16_t*>(z[1].data() + 64),
                          z[2].data(), reinterpret_cast<const int*>(z[3].data()),
                          (int)(z[3].size() / 4), n, nc_node_dim, mesh_scale, v_r2i, shift);
}

int asg_copy_decoded(asg_ctx* ctx, asg_particle* out)
{
    if (!ctx || !out) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    if (ctx->dec_n <= 0) return fail(ctx, ASG_ERR_STATE, "nothing decoded");
    CK(cudaSetDevice(ctx->device));
    const int n = ctx->dec_n;
    const ShellIn L = shell_in_layout(n);
    if (int r = grow(ctx, ctx->aos, sizeof(asg_particle) * (size_t)n)) return r;
    unsigned char* b = P<unsigned char>(ctx->sh_in);
    launch_pack_aos(nullptr, reinterpret_cast<float4*>(b + L.pos), reinterpret_cast<float4*>(b + L.vel),
                    reinterpret_cast<float*>(b + L.rk), nullptr, reinterpret_cast<int*>(b + L.igrp), n,
                    ctx->aos.p, ctx->s);
    CK(cudaMemcpyAsync(out, ctx->aos.p, sizeof(asg_particle) * (size_t)n, cudaMemcpyDeviceToHost,
                       ctx->s));
    return finish(ctx, "copy_decoded");
}

int asg_load_decoded_periodic(asg_ctx* ctx, float boxsize, float buffer_factor,
                              int* np_with_buffers, int* np_local_kept)
{
    if (!ctx) return ASG_ERR_ARG;
    if (ctx->dec_n <= 0) return fail(ctx, ASG_ERR_STATE, "nothing decoded");
    if (int r = check_shell(ctx, ctx->dec_n, boxsize, buffer_factor)) return r;
    CK(cudaSetDevice(ctx->device));
    ctx->loaded = false;
    return load_shell(ctx, ctx->dec_n, boxsize, buffer_factor, np_with_buffers, np_local_kept);
}

static int run_knn(asg_ctx* ctx)
{
    const TreeView t = tree_view(ctx);
    phase_begin(ctx, ASG_PH_KNN);
    launch_knn_t33(P<float4>(ctx->pos), t, P<float>(ctx->t33), P<float>(ctx->rk),
                   P<int>(ctx->idx33), P<int>(ctx->blist), ctx->d_err, ctx->s, ctx->knn_warps);
    phase_end(ctx);
    phase_begin(ctx, ASG_PH_TIES);  // only bundles with an exact tie at the 33rd distance
    launch_knn_ties(P<float4>(ctx->pos), t, P<float>(ctx->t33), P<int>(ctx->idx33), 0,
                    ctx->d_err, ctx->s);
    phase_end(ctx);
    ctx->idx33_all = false;
    ctx->rk_checked = false;
    ensure_rk_checked(ctx);
    phase_begin(ctx, ASG_PH_DENS);
    launch_dens(P<float4>(ctx->pos), t, P<float>(ctx->t33), P<int>(ctx->idx33), P<int>(ctx->blist),
                P<float>(ctx->rk), P<int>(ctx->dexp), P<unsigned long long>(ctx->dacc),
                P<float4>(ctx->vel), ctx->d_err, ctx->s);
    phase_end(ctx);
    ctx->knn_done = true;
    return 0;
}

int asg_run_neighbor_search(asg_ctx* ctx)
{
    if (!ctx) return ASG_ERR_ARG;
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    if (ctx->n < K_NN) return fail(ctx, ASG_ERR_FEW, "fewer than 33 particles");
    CK(cudaSetDevice(ctx->device));
    run_knn(ctx);
    int r = finish(ctx, "neighbor_search");
    if (r) ctx->knn_done = false;
    return r;
}

static int queue_mark(asg_ctx* ctx, const asg_halo* halos, int nh)
{
    if (nh <= 0) return 0;
    if (int r = grow(ctx, ctx->halos, sizeof(asg_halo) * (size_t)nh)) return r;
    if (int r = grow(ctx, ctx->hcount, sizeof(long long) * (size_t)nh)) return r;
    if (int r = grow(ctx, ctx->hmass, sizeof(double) * (size_t)nh)) return r;
    CK(cudaMemcpyAsync(ctx->halos.p, halos, sizeof(asg_halo) * (size_t)nh, cudaMemcpyHostToDevice,
                       ctx->s));
    phase_begin(ctx, ASG_PH_HALOS);
    launch_mark_halos(P<float4>(ctx->pos), tree_view(ctx), P<float>(ctx->halos), nh, ctx->left,
                      ctx->right, P<int>(ctx->igrp), P<long long>(ctx->hcount),
                      P<double>(ctx->hmass), ctx->s);
    phase_end(ctx);
    return 0;
}

static int collect_mark(asg_ctx* ctx, int nh, long* np_halo, double* m_halo)
{
    long tot = 0;
    double mh = 0.0;
    if (nh > 0) {
        std::vector<long long> cnt((size_t)nh);
        std::vector<double> m8((size_t)nh);
        CK(cudaMemcpy(cnt.data(), ctx->hcount.p, sizeof(long long) * (size_t)nh,
                      cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(m8.data(), ctx->hmass.p, sizeof(double) * (size_t)nh,
                      cudaMemcpyDeviceToHost));
        for (int i = 0; i < nh; ++i) {  // halo order, as the reference's serial loop
            if (cnt[(size_t)i] < 0) return fail(ctx, ASG_ERR_STACK, "mark_halos: stack overflow");
            tot += (long)cnt[(size_t)i];
            mh += m8[(size_t)i];
        }
    }
    if (np_halo) *np_halo = tot;
    if (m_halo) *m_halo = mh;
    return 0;
}

int asg_run_mark_halos(asg_ctx* ctx, const asg_halo* halos, int nh, long* np_halo, double* m_halo)
{
    if (!ctx || nh < 0 || (nh > 0 && !halos)) return fail(ctx, ASG_ERR_ARG, "bad halo list");
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    CK(cudaSetDevice(ctx->device));
    if (int r = queue_mark(ctx, halos, nh)) return r;
    if (int r = finish(ctx, "mark_halos")) return r;
    return collect_mark(ctx, nh, np_halo, m_halo);
}

int asg_run_fof(asg_ctx* ctx, float ll, int* ngroup)
{
    if (!ctx || !ngroup || !(ll >= 0.0f) || !std::isfinite(ll))
        return fail(ctx, ASG_ERR_ARG, "bad FOF arguments");
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    CK(cudaSetDevice(ctx->device));
    const int n = ctx->n;
    if (int r = grow(ctx, ctx->uf, 4 * (size_t)n)) return r;
    if (int r = grow(ctx, ctx->minin, 4 * (size_t)n)) return r;
    if (int r = grow(ctx, ctx->mark, 4 * ((size_t)n + 1))) return r;
    if (int r = grow(ctx, ctx->scan_tmp, scan_temp_bytes((size_t)n + 1))) return r;
    phase_begin(ctx, ASG_PH_FOF);
    launch_iota(P<int>(ctx->uf), n, ctx->s);
    CK(cudaMemsetAsync(ctx->minin.p, 0x7f, 4 * (size_t)n, ctx->s));
    CK(cudaMemsetAsync(ctx->mark.p, 0, 4 * ((size_t)n + 1), ctx->s));
    launch_fof_link(P<float4>(ctx->pos), tree_view(ctx), ll, P<int>(ctx->uf), ctx->d_err, ctx->s);
    launch_fof_finish(P<float4>(ctx->pos), n, P<int>(ctx->uf), P<int>(ctx->minin), P<int>(ctx->mark),
                      ctx->s);
    exclusive_scan_u32(P<uint32_t>(ctx->mark), (size_t)n + 1, ctx->scan_tmp.p, ctx->s);
    launch_fof_label(P<float4>(ctx->pos), n, P<int>(ctx->uf), P<int>(ctx->minin),
                     P<uint32_t>(ctx->mark), P<int>(ctx->igrp), ctx->s);
    phase_end(ctx);
    uint32_t ng = 0;
    CK(cudaMemcpyAsync(&ng, P<uint32_t>(ctx->mark) + n, 4, cudaMemcpyDeviceToHost, ctx->s));
    if (int r = finish(ctx, "fof")) return r;
    *ngroup = (int)ng;
    return 0;
}

__global__ static void k_label_range(const int* igrp, int n, int ngrp, int* err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && (igrp[i] < 0 || igrp[i] > ngrp)) atomicOr(err, ERR_RANGE);
}

int asg_run_remove_small_groups(asg_ctx* ctx, int ngrp, int* nhalo)
{
    if (!ctx || !nhalo || ngrp < 0) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    if (ngrp > ctx->n) return fail(ctx, ASG_ERR_ARG, "ngrp larger than the particle count");
    CK(cudaSetDevice(ctx->device));
    const int n = ctx->n;
    const size_t nl = (size_t)ngrp + 2;
    if (int r = grow(ctx, ctx->lab_cnt, 4 * nl)) return r;
    if (int r = grow(ctx, ctx->lab_scan, 4 * nl)) return r;
    if (int r = grow(ctx, ctx->scan_tmp, scan_temp_bytes(nl))) return r;
    k_label_range<<<(n + 255) / 256, 256, 0, ctx->s>>>(P<int>(ctx->igrp), n, ngrp, ctx->d_err);
    count_launches(1);
    if (int r = finish(ctx, "remove_small_groups")) {
        return fail(ctx, r == ASG_ERR_RANGE ? ASG_ERR_ARG : r, "group labels outside [0, ngrp]");
    }
    CK(cudaMemsetAsync(ctx->lab_cnt.p, 0, 4 * nl, ctx->s));
    launch_count_labels(P<int>(ctx->igrp), n, P<uint32_t>(ctx->lab_cnt), ctx->s);
    launch_keep_mask(P<uint32_t>(ctx->lab_cnt), ngrp, 20, ctx->s);  // threshold, fof.cpp:107
    CK(cudaMemsetAsync(P<uint32_t>(ctx->lab_cnt) + ngrp + 1, 0, 4, ctx->s));
    CK(cudaMemcpyAsync(ctx->lab_scan.p, ctx->lab_cnt.p, 4 * nl, cudaMemcpyDeviceToDevice, ctx->s));
    exclusive_scan_u32(P<uint32_t>(ctx->lab_scan), nl, ctx->scan_tmp.p, ctx->s);
    launch_relabel(P<int>(ctx->igrp), n, P<uint32_t>(ctx->lab_scan), P<uint32_t>(ctx->lab_cnt),
                   ctx->s);
    uint32_t nh = 0;
    CK(cudaMemcpyAsync(&nh, P<uint32_t>(ctx->lab_scan) + ngrp + 1, 4, cudaMemcpyDeviceToHost,
                       ctx->s));
    if (int r = finish(ctx, "remove_small_groups")) return r;
    *nhalo = (int)nh;
    return 0;
}

// cap == 0: size the pair arrays from the pair count (one host synchronisation);
// cap > 0: pair arrays of that capacity, no synchronisation (stream capture)
static int queue_deposit(asg_ctx* ctx, float boxsize, const int* ncs, int n_nc, int sign,
                         int periodic, const int* coords, int density_only, uint32_t cap = 0)
{
    if (!ncs || n_nc <= 0 || n_nc > MAX_MESHES) return fail(ctx, ASG_ERR_ARG, "1..8 meshes");
    if (!(boxsize > 0.0f) || !std::isfinite(boxsize)) return fail(ctx, ASG_ERR_ARG, "boxsize");
    for (int k = 0; k < n_nc; ++k)
        if (ncs[k] <= 0 || ncs[k] > 1290) return fail(ctx, ASG_ERR_ARG, "nc out of range");
    ensure_rk_checked(ctx);
    if ((int)ctx->meshes.size() < n_nc) ctx->meshes.resize((size_t)n_nc);
    ctx->mesh_boxsize = boxsize;
    DepositParams p;
    std::memset(&p, 0, sizeof(p));
    p.n_jobs = n_nc;
    p.boxsize = boxsize;
    p.rbox = 1.0f / boxsize;  // correctly rounded (IEEE float division on the host)
    p.sign = sign;
    p.periodic = periodic ? 1 : 0;
    p.density_only = density_only ? 1 : 0;
    p.seg = ctx->dep_seg;
    p.mma = ctx->dep_mma;
    for (int d = 0; d < 3; ++d) p.offset[d] = periodic && coords ? boxsize * (float)coords[d] : 0.0f;
    int tiles = 0;
    for (int k = 0; k < n_nc; ++k) {
        MeshBuf& mb = ctx->meshes[(size_t)k];
        const int nc = ncs[k];
        const size_t nm = (size_t)nc * nc * nc * (density_only ? 1 : 6);
        const int tpd = (nc + 7) / 8;
        if (int r = grow(ctx, mb.mesh, 4 * nm)) return r;
        if (int r = grow(ctx, mb.partial, 16 * (size_t)tpd * tpd * tpd)) return r;
        mb.nc = nc;
        mb.words = nm;
        MeshJob& j = p.job[k];
        j.nc = nc;
        j.dx = boxsize / nc;  // float / int, as coarse_mesh.cpp:58
        j.ncf = (float)nc;
        j.tiles[0] = j.tiles[1] = j.tiles[2] = tpd;
        j.tile_begin = tiles;
        j.mesh = P<float>(mb.mesh);
        j.partial = P<double>(mb.partial);
        tiles += tpd * tpd * tpd;
    }
    if (int r = grow(ctx, ctx->totals, 16 * (size_t)n_nc)) return r;
    // the tiles' processing order, cached while the meshes stay the same (a
    // captured call without it takes the tiles in tile order: the same sums)
    const std::vector<int> okey(ncs, ncs + n_nc);
    if (ctx->dep_order_on && okey != ctx->dep_order_key && !cap) {
        if (int r = grow(ctx, ctx->dep_order, 8 * (size_t)tiles)) return r;
        std::vector<uint32_t> h(2 * (size_t)tiles);
        deposit_tile_order(p, tiles, h.data());
        CK(cudaMemcpyAsync(ctx->dep_order.p, h.data(), 8 * (size_t)tiles, cudaMemcpyHostToDevice,
                           ctx->s));
        CK(cudaStreamSynchronize(ctx->s));
        ctx->dep_order_key = okey;
    }
    if (ctx->dep_order_on && okey == ctx->dep_order_key) {
        p.order = P<uint32_t>(ctx->dep_order);
        p.pos = p.order + tiles;
    }
    // particle records and pair counts, then size the pair arrays
    const int n = ctx->n;
    const size_t T1 = (size_t)tiles + 1;
    if (int r = grow(ctx, ctx->dep_rec, deposit_prep_bytes(n))) return r;
    if (int r = grow(ctx, ctx->dep_pcount, 4 * ((size_t)n + 1) + scan_temp_bytes((size_t)n + 1)))
        return r;
    if (int r = grow(ctx, ctx->dep_tiles, deposit_tile_bytes(tiles))) return r;
    if (int r = grow(ctx, ctx->dep_counter, 16)) return r;
    DepositScratch w;
    w.rec = P<float4>(ctx->dep_rec);
    w.pcount = P<uint32_t>(ctx->dep_pcount);
    w.scan_tmp_n = (void*)(w.pcount + n + 1);
    w.tstart = P<uint32_t>(ctx->dep_tiles);
    w.tcount = w.tstart + T1;
    w.item_off = w.tcount + T1;
    w.scan_tmp_t = (void*)(w.item_off + T1);
    w.next_item = P<int>(ctx->dep_counter);
    phase_begin(ctx, ASG_PH_DEPOSIT);
    launch_deposit_prep(P<float4>(ctx->pos), P<float4>(ctx->vel), P<int>(ctx->igrp),
                        P<float>(ctx->rk), n, p, w, ctx->d_err, ctx->s);
    uint32_t npairs = cap;
    if (!cap) {
        if (int r = read_words(ctx, w.pcount + n)) return r;
        npairs = ctx->h_u32[0];
    }
    const size_t NP = (size_t)npairs + 1;
    if (int r = grow(ctx, ctx->dep_pairs, 16 * NP)) return r;
    if (int r = grow(ctx, ctx->dep_sort, radix_sort_temp_bytes((int)NP))) return r;
    const uint32_t max_items = deposit_max_items(tiles, npairs, p.seg);
    if (int r = grow(ctx, ctx->dep_partial, deposit_partial_bytes(max_items) + 16)) return r;
    w.keys0 = P<uint32_t>(ctx->dep_pairs);
    w.keys1 = w.keys0 + NP;
    w.vals0 = reinterpret_cast<int*>(w.keys1 + NP);
    w.vals1 = w.vals0 + NP;
    w.sort_tmp = ctx->dep_sort.p;
    w.partial = P<float>(ctx->dep_partial);
    if (!cap) ctx->dep_npairs = npairs;
    ctx->dep_tiles_n = tiles;
    launch_deposit_run(n, p, tiles, npairs, cap != 0, w, ctx->d_err, ctx->s);
    for (int k = 0; k < n_nc; ++k) {
        const int tpd = (ncs[k] + 7) / 8;
        launch_reduce_partials(P<double>(ctx->meshes[(size_t)k].partial), tpd * tpd * tpd,
                               P<double>(ctx->totals) + 2 * k, ctx->s);
    }
    phase_end(ctx);
    return 0;
}

// The meshes of an end-to-end call to the host, on the output stream after the
// deposit (timed as the output phase: from the end of the deposit until the
// copies are done).  Depositing the meshes one at a time to overlap their
// copies with the next deposit was measured and dropped: the three deposits
// cost 3.6 ms more than one on the 256^3 step, the copies about 2.
static int queue_mesh_out(asg_ctx* ctx, int n_nc, float* const* meshes)
{
    phase_begin(ctx, ASG_PH_OUTPUT);
    CK(cudaEventRecord(ctx->fields_ready, ctx->s));
    CK(cudaStreamWaitEvent(ctx->s_out, ctx->fields_ready, 0));
    for (int k = 0; k < n_nc; ++k)
        if (meshes && meshes[k])
            CK(cudaMemcpyAsync(meshes[k], ctx->meshes[(size_t)k].mesh.p,
                               4 * ctx->meshes[(size_t)k].words, cudaMemcpyDeviceToHost, ctx->s_out));
    if (ctx->timing) {
        cudaEvent_t e = next_event(ctx);
        cudaEventRecord(e, ctx->s_out);
        cudaStreamWaitEvent(ctx->s, e, 0);
    }
    phase_end(ctx);
    return 0;
}

int asg_run_deposit(asg_ctx* ctx, float boxsize, const int* ncs, int n_nc, int sign,
                    int periodic, const int* coords, int density_only, double* totals)
{
    if (!ctx) return ASG_ERR_ARG;
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    CK(cudaSetDevice(ctx->device));
    if (int r = queue_deposit(ctx, boxsize, ncs, n_nc, sign, periodic, coords, density_only))
        return r;
    if (totals)
        CK(cudaMemcpyAsync(totals, ctx->totals.p, 16 * (size_t)n_nc, cudaMemcpyDeviceToHost, ctx->s));
    return finish(ctx, "deposit");
}

float* asg_mesh_device(asg_ctx* ctx, int k)
{
    if (!ctx || k < 0 || k >= (int)ctx->meshes.size()) return nullptr;
    return P<float>(ctx->meshes[(size_t)k].mesh);
}

int asg_copy_mesh(asg_ctx* ctx, int k, float* host)
{
    if (!ctx || !host || k < 0 || k >= (int)ctx->meshes.size() || !ctx->meshes[(size_t)k].nc)
        return fail(ctx, ASG_ERR_ARG, "no such mesh");
    CK(cudaMemcpyAsync(host, ctx->meshes[(size_t)k].mesh.p, 4 * ctx->meshes[(size_t)k].words,
                       cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return 0;
}

int asg_run_normalise(asg_ctx* ctx, int k)
{
    if (!ctx || k < 0 || k >= (int)ctx->meshes.size() || !ctx->meshes[(size_t)k].nc)
        return fail(ctx, ASG_ERR_ARG, "no such mesh");
    const MeshBuf& mb = ctx->meshes[(size_t)k];
    if (mb.words != 6 * (size_t)mb.nc * mb.nc * mb.nc)
        return fail(ctx, ASG_ERR_STATE, "density-only mesh has no c/v channels");
    CK(cudaSetDevice(ctx->device));
    const float vol = std::pow(ctx->mesh_boxsize / mb.nc, 3.0f);  // coarse_mesh.cpp:151
    launch_normalise(P<float>(ctx->meshes[(size_t)k].mesh), mb.nc, vol, ctx->s);
    return finish(ctx, "normalise");
}

int asg_store_particles(asg_ctx* ctx, asg_particle* p)
{
    if (!ctx || !p) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    CK(cudaSetDevice(ctx->device));
    if (int r = grow(ctx, ctx->aos, sizeof(asg_particle) * (size_t)ctx->n)) return r;
    launch_pack_aos(ctx->perm, P<float4>(ctx->pos), P<float4>(ctx->vel), P<float>(ctx->rk), nullptr,
                    P<int>(ctx->igrp), ctx->n, ctx->aos.p, ctx->s);
    CK(cudaMemcpyAsync(p, ctx->aos.p, sizeof(asg_particle) * (size_t)ctx->n, cudaMemcpyDeviceToHost,
                       ctx->s));
    return finish(ctx, "store");
}

__global__ static void k_dens_of(const float4* vel, int n, float* dens)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dens[i] = vel[i].w;
}

int asg_store_fields_device(asg_ctx* ctx, float* d_rk, float* d_dens, int* d_igrp)
{
    if (!ctx) return ASG_ERR_ARG;
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    CK(cudaSetDevice(ctx->device));
    float* dens_s = nullptr;
    if (d_dens) {  // sorted dens lives in vel.w: stage it in a scratch array
        if (int r = grow(ctx, ctx->lab_scan, 4 * (size_t)ctx->n)) return r;
        dens_s = P<float>(ctx->lab_scan);
        k_dens_of<<<(ctx->n + 255) / 256, 256, 0, ctx->s>>>(P<float4>(ctx->vel), ctx->n, dens_s);
        count_launches(1);
    }
    launch_scatter_fields(ctx->perm, P<float>(ctx->rk), dens_s, P<int>(ctx->igrp), ctx->n, d_rk,
                          d_dens, d_igrp, ctx->s);
    return finish(ctx, "store_fields");
}

int asg_get_knn(asg_ctx* ctx, float* t33, int* idx33)
{
    if (!ctx) return ASG_ERR_ARG;
    if (!ctx->knn_done) return fail(ctx, ASG_ERR_STATE, "no neighbour search done");
    CK(cudaSetDevice(ctx->device));
    const size_t n = (size_t)ctx->n;
    if (int r = grow(ctx, ctx->uf, 4 * n)) return r;
    if (int r = grow(ctx, ctx->minin, 4 * n)) return r;
    if (!ctx->idx33_all) {  // the hot path resolves idx33 only where the 33rd value is tied
        launch_knn_ties(P<float4>(ctx->pos), tree_view(ctx), P<float>(ctx->t33),
                        P<int>(ctx->idx33), 1, ctx->d_err, ctx->s);
        ctx->idx33_all = true;
    }
    launch_scatter_fields(ctx->perm, P<float>(ctx->t33), nullptr, P<int>(ctx->idx33), ctx->n,
                          P<float>(ctx->uf), nullptr, P<int>(ctx->minin), ctx->s);
    if (t33) CK(cudaMemcpyAsync(t33, ctx->uf.p, 4 * n, cudaMemcpyDeviceToHost, ctx->s));
    if (idx33) CK(cudaMemcpyAsync(idx33, ctx->minin.p, 4 * n, cudaMemcpyDeviceToHost, ctx->s));
    return finish(ctx, "get_knn");
}

// ---- reference-shaped one-shot calls --------------------------------------------

int asg_neighbor_search(asg_ctx* ctx, asg_particle* p, int np, float left, float right)
{
    if (np < K_NN && np > 0) return fail(ctx, ASG_ERR_FEW, "fewer than 33 particles");
    if (int r = asg_load_particles(ctx, p, np, left, right)) return r;
    if (int r = asg_run_neighbor_search(ctx)) return r;
    return asg_store_particles(ctx, p);
}

// load for calls whose reference signature carries no cube bounds: the key
// grid only orders particles, so it spans the particles' own bounding cube,
// found on the device
static int load_for_deposit(asg_ctx* ctx, const asg_particle* p, int np)
{
    if (!ctx || !p || np <= 0) return fail(ctx, ASG_ERR_ARG, "null argument or np <= 0");
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    if (int r = grow(ctx, ctx->aos, sizeof(asg_particle) * (size_t)np)) return r;
    if (int r = grow(ctx, ctx->lohi, 8)) return r;
    ctx->n = np;
    ctx->left = -INFINITY;
    ctx->right = INFINITY;
    phase_begin(ctx, ASG_PH_UPLOAD);
    CK(cudaMemcpyAsync(ctx->aos.p, p, sizeof(asg_particle) * (size_t)np, cudaMemcpyHostToDevice,
                       ctx->s));
    phase_end(ctx);
    phase_begin(ctx, ASG_PH_INDEX);
    launch_unpack_aos(ctx->aos.p, np, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                      P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    launch_space_keys(P<float4>(ctx->pos_in), np, 0.0f, 0.0f, P<int>(ctx->lohi), 0,
                  P<uint64_t>(ctx->keys0), P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
    int r = finish(ctx, "load");
    if (r) ctx->loaded = false;
    return r;
}

int asg_assign_on_meshes(asg_ctx* ctx, const asg_particle* p, int np, float boxsize,
                         const int* ncs, int n_nc, int sign, int periodic, const int* coords,
                         float* const* meshes, double* totals)
{
    if (!meshes) return fail(ctx, ASG_ERR_ARG, "null meshes");
    if (int r = load_for_deposit(ctx, p, np)) return r;
    if (int r = asg_run_deposit(ctx, boxsize, ncs, n_nc, sign, periodic, coords, 0, totals))
        return r;
    for (int k = 0; k < n_nc; ++k)
        if (meshes[k])
            if (int r = asg_copy_mesh(ctx, k, meshes[k])) return r;
    return 0;
}

int asg_assign_on_mesh(asg_ctx* ctx, const asg_particle* p, int np, float boxsize, int nc,
                       int sign, float* mesh, double* totals)
{
    float* m[1] = {mesh};
    return asg_assign_on_meshes(ctx, p, np, boxsize, &nc, 1, sign, 0, nullptr, m, totals);
}

int asg_assign_on_density_mesh(asg_ctx* ctx, const asg_particle* p, int np, float boxsize,
                               int nc, int sign, float* mesh)
{
    if (!mesh) return fail(ctx, ASG_ERR_ARG, "null mesh");
    if (int r = load_for_deposit(ctx, p, np)) return r;
    if (int r = asg_run_deposit(ctx, boxsize, &nc, 1, sign, 0, nullptr, 1, nullptr)) return r;
    return asg_copy_mesh(ctx, 0, mesh);
}

int asg_normalise_mesh(asg_ctx* ctx, float* mesh, int nc, float boxsize)
{
    if (!ctx || !mesh || nc <= 0 || nc > 1290) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    const size_t words = 6 * (size_t)nc * nc * nc;
    if (int r = grow(ctx, ctx->aos, 4 * words)) return r;
    const float vol = std::pow(boxsize / nc, 3.0f);  // pow(float, float) as coarse_mesh.cpp:151
    CK(cudaMemcpyAsync(ctx->aos.p, mesh, 4 * words, cudaMemcpyHostToDevice, ctx->s));
    launch_normalise(P<float>(ctx->aos), nc, vol, ctx->s);
    CK(cudaMemcpyAsync(mesh, ctx->aos.p, 4 * words, cudaMemcpyDeviceToHost, ctx->s));
    return finish(ctx, "normalise");
}

int asg_group_fof(asg_ctx* ctx, asg_particle* p, int np, float left, float right, float ll,
                  int* ngroup)
{
    if (int r = asg_load_particles(ctx, p, np, left, right)) return r;
    if (int r = asg_run_fof(ctx, ll, ngroup)) return r;
    return asg_store_particles(ctx, p);
}

int asg_remove_small_groups(asg_ctx* ctx, asg_particle* p, int np, int ngrp, int* nhalo)
{
    if (int r = load_for_deposit(ctx, p, np)) return r;
    if (int r = asg_run_remove_small_groups(ctx, ngrp, nhalo)) return r;
    return asg_store_particles(ctx, p);
}

int asg_mark_halo_particles(asg_ctx* ctx, asg_particle* p, int np, const asg_halo* halos,
                            int nh, float left, float right, long* np_halo, double* m_halo)
{
    if (int r = asg_load_particles(ctx, p, np, left, right)) return r;
    if (int r = asg_run_mark_halos(ctx, halos, nh, np_halo, m_halo)) return r;
    return asg_store_particles(ctx, p);
}

// ---- outputs ----------------------------------------------------------------------

// FOF catalogue on device arrays indexed by j; records and count back to the host
static int run_catalogue(asg_ctx* ctx, const float4* pos, const float4* vel, const int* igrp, int n,
                         int w_index, int nhalo, float boxsize, asg_fof_halo* out, int* nlocal)
{
    const size_t rec_bytes = sizeof(asg_fof_halo) * (size_t)(nhalo > 0 ? nhalo : 1);
    const size_t o_cnt = (rec_bytes + 15) & ~size_t(15);
    if (int r = grow(ctx, ctx->cat, fof_catalogue_bytes(n, nhalo))) return r;
    if (int r = grow(ctx, ctx->cat_out, o_cnt + 16)) return r;
    unsigned char* ob = P<unsigned char>(ctx->cat_out);
    CK(cudaMemsetAsync(ob, 0, o_cnt + 16, ctx->s));
    launch_fof_catalogue(pos, vel, igrp, n, w_index, nhalo, boxsize, ctx->cat.p,
                         reinterpret_cast<float*>(ob), reinterpret_cast<uint32_t*>(ob + o_cnt), ctx->s);
    if (nhalo > 0) CK(cudaMemcpyAsync(out, ob, sizeof(asg_fof_halo) * (size_t)nhalo,
                                      cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaMemcpyAsync(ctx->h_u32, ob + o_cnt, 4, cudaMemcpyDeviceToHost, ctx->s));
    if (int r = finish(ctx, "fof_halos")) return r;
    *nlocal = (int)ctx->h_u32[0];
    return ASG_OK;
}

int asg_fof_halos(asg_ctx* ctx, const asg_particle* p, int np, int nhalo, float boxsize,
                  asg_fof_halo* out, int* nlocal)
{
    if (!ctx || !p || !nlocal || (nhalo > 0 && !out) || np <= 0 || nhalo < 0 || nhalo > np)
        return fail(ctx, ASG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    const size_t n = (size_t)np;
    // staging buffers only: a loaded particle set stays valid
    int r = grow(ctx, ctx->aos, sizeof(asg_particle) * n);
    if (!r) r = grow(ctx, ctx->pos_in, 16 * n);
    if (!r) r = grow(ctx, ctx->vel_in, 16 * n);
    if (!r) r = grow(ctx, ctx->igrp_in, 4 * n);
    if (!r) r = grow(ctx, ctx->rk_in, 4 * n);
    if (r) return r;
    CK(cudaMemcpyAsync(ctx->aos.p, p, sizeof(asg_particle) * n, cudaMemcpyHostToDevice, ctx->s));
    launch_unpack_aos(ctx->aos.p, np, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                      P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    return run_catalogue(ctx, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in), P<int>(ctx->igrp_in),
                         np, 0, nhalo, boxsize, out, nlocal);
}

int asg_run_fof_halos(asg_ctx* ctx, int nhalo, float boxsize, asg_fof_halo* out, int* nlocal)
{
    if (!ctx || !nlocal || (nhalo > 0 && !out) || nhalo < 0) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    if (!ctx->loaded) return fail(ctx, ASG_ERR_STATE, "no particle set loaded");
    if (nhalo > ctx->n) return fail(ctx, ASG_ERR_ARG, "nhalo larger than the particle count");
    CK(cudaSetDevice(ctx->device));
    return run_catalogue(ctx, P<float4>(ctx->pos), P<float4>(ctx->vel), P<int>(ctx->igrp), ctx->n, 1,
                         nhalo, boxsize, out, nlocal);
}

int asg_write_fof_halos(asg_ctx* ctx, const char* filename, const asg_particle* p, int np,
                        int nhalo, float boxsize)
{
    if (!filename) return fail(ctx, ASG_ERR_ARG, "null file name");
    std::vector<asg_fof_halo> rec((size_t)(nhalo > 0 ? nhalo : 1));
    int nl = 0;
    if (int r = asg_fof_halos(ctx, p, np, nhalo, boxsize, rec.data(), &nl)) return r;
    if (int r = write_fof_file(filename, reinterpret_cast<const float*>(rec.data()), nl))
        return fail(ctx, r, std::string("cannot write ") + filename);
    return ASG_OK;
}

int asg_write_mesh_separate(asg_ctx* ctx, const char* base, int inode, float* mesh, int nc,
                            float boxsize)
{
    if (!base) return fail(ctx, ASG_ERR_ARG, "null base name");
    if (int r = asg_normalise_mesh(ctx, mesh, nc, boxsize)) return r;
    if (int r = write_mesh_files(base, inode, mesh, nc))
        return fail(ctx, r, std::string("cannot write mesh files at ") + base);
    return ASG_OK;
}

int asg_write_mesh_device(asg_ctx* ctx, int k, const char* base, int inode)
{
    if (!base) return fail(ctx, ASG_ERR_ARG, "null base name");
    if (int r = asg_run_normalise(ctx, k)) return r;
    const MeshBuf& mb = ctx->meshes[(size_t)k];
    std::vector<float> host(mb.words);
    if (int r = asg_copy_mesh(ctx, k, host.data())) return r;
    if (int r = write_mesh_files(base, inode, host.data(), mb.nc))
        return fail(ctx, r, std::string("cannot write mesh files at ") + base);
    return ASG_OK;
}

int asg_set_timing(asg_ctx* ctx, int enable)
{
    if (!ctx) return ASG_ERR_ARG;
    ctx->timing = enable != 0;
    for (double& m : ctx->phase_ms) m = 0.0;
    return ASG_OK;
}

int asg_phase_ms(asg_ctx* ctx, double* ms)
{
    if (!ctx || !ms) return ASG_ERR_ARG;
    for (int i = 0; i < ASG_NPHASES; ++i) ms[i] = ctx->phase_ms[i];
    return ASG_OK;
}

const char* asg_phase_name(int phase)
{
    static const char* names[ASG_NPHASES] = {"index", "knn_t33", "knn_ties", "check_rk", "dens",
                                             "deposit", "halos", "fof", "upload", "output"};
    return (phase >= 0 && phase < ASG_NPHASES) ? names[phase] : "?";
}

__global__ static void k_fma_probe(float* out, int iters, float a, float b)
{
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3f + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int asg_deposit_stats(asg_ctx* ctx, long long* pairs, long long* tiles, long long* items)
{
    if (!ctx) return ASG_ERR_ARG;
    if (!ctx->dep_counter.p) return fail(ctx, ASG_ERR_STATE, "no deposit run yet");
    CK(cudaSetDevice(ctx->device));
    uint32_t it = 0;
    const uint32_t* item_off = P<uint32_t>(ctx->dep_tiles) + 2 * ((size_t)ctx->dep_tiles_n + 1);
    CK(cudaMemcpy(&it, item_off + ctx->dep_tiles_n, 4, cudaMemcpyDeviceToHost));
    if (pairs) *pairs = ctx->dep_npairs;
    if (tiles) *tiles = ctx->dep_tiles_n;
    if (items) *items = it;
    return ASG_OK;
}

int asg_measure_fp32_peak(asg_ctx* ctx, double* tflops)
{
    if (!ctx || !tflops) return ASG_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    if (int r = grow(ctx, ctx->lab_scan, sizeof(float) * (size_t)blocks * threads)) return r;
    cudaEvent_t e0 = next_event(ctx), e1 = next_event(ctx);
    k_fma_probe<<<blocks, threads, 0, ctx->s>>>(P<float>(ctx->lab_scan), iters / 8, 0.9999f, 1e-4f);
    CK(cudaEventRecord(e0, ctx->s));
    k_fma_probe<<<blocks, threads, 0, ctx->s>>>(P<float>(ctx->lab_scan), iters, 0.9999f, 1e-4f);
    CK(cudaEventRecord(e1, ctx->s));
    count_launches(2);
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    ctx->ev_used = 0;
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return finish(ctx, "fp32_peak");
}

int asg_smooth(asg_ctx* ctx, asg_particle* p, int np, float left, float right, float boxsize,
               const asg_halo* halos, int nh, const int* ncs, int n_nc, int sign,
               float* const* meshes, double* totals, long* np_halo, double* m_halo)
{
    if (!ctx || !p || (nh > 0 && !halos) || nh < 0) return fail(ctx, ASG_ERR_ARG, "bad arguments");
    if (np < K_NN) return fail(ctx, np > 0 ? ASG_ERR_FEW : ASG_ERR_ARG, "fewer than 33 particles");
    if (int r = check_bounds(ctx, np, left, right)) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    if (int r = grow(ctx, ctx->aos, sizeof(asg_particle) * (size_t)np)) return r;
    ctx->n = np;
    ctx->left = left;
    ctx->right = right;
    phase_begin(ctx, ASG_PH_UPLOAD);
    CK(cudaMemcpyAsync(ctx->aos.p, p, sizeof(asg_particle) * (size_t)np, cudaMemcpyHostToDevice,
                       ctx->s));
    phase_end(ctx);
    phase_begin(ctx, ASG_PH_INDEX);
    launch_unpack_aos(ctx->aos.p, np, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                      P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    launch_space_keys(P<float4>(ctx->pos_in), np, left, right, nullptr, 0, P<uint64_t>(ctx->keys0),
                  P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
    run_knn(ctx);
    if (int r = queue_mark(ctx, halos, nh)) return r;
    // rk, dens and igrp are final: copy the records out while the deposit runs
    CK(cudaEventRecord(ctx->fields_ready, ctx->s));
    CK(cudaStreamWaitEvent(ctx->s_out, ctx->fields_ready, 0));
    launch_pack_aos(ctx->perm, P<float4>(ctx->pos), P<float4>(ctx->vel), P<float>(ctx->rk), nullptr,
                    P<int>(ctx->igrp), np, ctx->aos.p, ctx->s_out);
    CK(cudaMemcpyAsync(p, ctx->aos.p, sizeof(asg_particle) * (size_t)np, cudaMemcpyDeviceToHost,
                       ctx->s_out));
    const int rd = queue_deposit(ctx, boxsize, ncs, n_nc, sign, 0, nullptr, 0);
    if (!rd) queue_mesh_out(ctx, n_nc, meshes);
    CK(cudaStreamSynchronize(ctx->s_out));  // the records and meshes are out before any return
    if (rd) return rd;
    if (totals)
        CK(cudaMemcpyAsync(totals, ctx->totals.p, 16 * (size_t)n_nc, cudaMemcpyDeviceToHost, ctx->s));
    if (int r = finish(ctx, "smooth")) return r;
    return collect_mark(ctx, nh, np_halo, m_halo);
}

int asg_smooth_quantised(asg_ctx* ctx, const int* cell, const uint16_t* off, const float* v,
                         int np, float left, float right, float cell_size, int grid, float boxsize,
                         const int* ncs, int n_nc, int sign, float* rk, float* dens,
                         float* const* meshes, double* totals)
{
    if (!ctx || !cell || !off) return fail(ctx, ASG_ERR_ARG, "null argument");
    if (np < K_NN) return fail(ctx, np > 0 ? ASG_ERR_FEW : ASG_ERR_ARG, "fewer than 33 particles");
    if (int r = check_bounds(ctx, np, left, right)) return r;
    if (int r = check_quant(ctx, grid, cell_size, left, right)) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, np)) return r;
    const size_t n = (size_t)np;
    if (int r = grow(ctx, ctx->uf, 4 * n)) return r;
    if (int r = grow(ctx, ctx->minin, 4 * n)) return r;
    if (int r = grow(ctx, ctx->lab_scan, 4 * n)) return r;
    const int* dc = nullptr;
    const uint16_t* doff = nullptr;
    const float* dv = nullptr;
    phase_begin(ctx, ASG_PH_UPLOAD);
    if (int r = stage_quant(ctx, cell, off, v, np, &dc, &doff, &dv)) return r;
    phase_end(ctx);
    load_quant_device(ctx, dc, doff, dv, np, left, right, cell_size, grid);
    run_knn(ctx);
    // rk and dens are final: back to input order and out while the deposit runs
    CK(cudaEventRecord(ctx->fields_ready, ctx->s));
    CK(cudaStreamWaitEvent(ctx->s_out, ctx->fields_ready, 0));
    k_dens_of<<<(np + 255) / 256, 256, 0, ctx->s_out>>>(P<float4>(ctx->vel), np,
                                                         P<float>(ctx->lab_scan));
    count_launches(1);
    launch_scatter_fields(ctx->perm, P<float>(ctx->rk), P<float>(ctx->lab_scan), nullptr, np,
                          P<float>(ctx->uf), P<float>(ctx->minin), nullptr, ctx->s_out);
    if (rk) CK(cudaMemcpyAsync(rk, ctx->uf.p, 4 * n, cudaMemcpyDeviceToHost, ctx->s_out));
    if (dens) CK(cudaMemcpyAsync(dens, ctx->minin.p, 4 * n, cudaMemcpyDeviceToHost, ctx->s_out));
    const int rd = queue_deposit(ctx, boxsize, ncs, n_nc, sign, 0, nullptr, 0);
    if (!rd) queue_mesh_out(ctx, n_nc, meshes);
    CK(cudaStreamSynchronize(ctx->s_out));  // rk, dens and the meshes are out before any return
    if (rd) return rd;
    if (totals)
        CK(cudaMemcpyAsync(totals, ctx->totals.p, 16 * (size_t)n_nc, cudaMemcpyDeviceToHost, ctx->s));
    return finish(ctx, "smooth_quantised");
}

}  // extern "C"

// ---- batched form: many cubes, one CUDA graph ------------------------------------------

struct asg_batch {
    asg_ctx* ctx = nullptr;
    int n_items = 0, n_nc = 0, sign = -1;
    std::vector<int> np, np_local, ncs;
    std::vector<float> left, right, box;
    std::vector<size_t> off;       // first particle of each item in the concatenated arrays
    std::vector<size_t> mesh_off;  // first float of mesh (item, k) in out_mesh
    size_t n_total = 0, mesh_words = 0;
    int max_n = 0;
    Buf in_x, in_v, out_rk, out_dens, out_mesh, out_tot;
    // mixed-precision items: int32 cell index and 3 x uint16 offsets per
    // particle (allocated with the first such item); quant[i] > 0 is item i's
    // grid, with its cell size in cell_size[i]
    Buf in_cell, in_off;
    std::vector<int> quant;
    std::vector<float> cell_size;
    std::vector<uint32_t> cap;     // pair capacity per item (from the planning pass)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;        // kernels per graph launch
    double last_ms = 0.0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // concurrent streams: item i runs on sub[i % sub.size()]; sub[0] is ctx, the
    // others are contexts of the batch (own stream and scratch) joined in the graph
    std::vector<asg_ctx*> sub;
    std::vector<cudaEvent_t> fork, join;
};

namespace {

void batch_drop_graph(asg_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// one item's whole path on the stream of ctx (the batch's context or one of its
// sub-contexts); cap = 0 sizes the deposit from its pair count (one
// synchronisation), cap > 0 synchronises nowhere
int batch_queue_item(asg_batch* b, asg_ctx* ctx, int i, uint32_t cap)
{
    const int n = b->np[(size_t)i];
    const size_t o = b->off[(size_t)i];
    ctx->n = n;
    ctx->left = b->left[(size_t)i];
    ctx->right = b->right[(size_t)i];
    if (b->quant[(size_t)i] > 0)
        launch_unpack_quant(P<int>(b->in_cell) + o, P<uint16_t>(b->in_off) + 3 * o,
                            P<float>(b->in_v) + 3 * o, n, b->quant[(size_t)i], ctx->left,
                            b->cell_size[(size_t)i], P<float4>(ctx->pos_in), P<float4>(ctx->vel_in),
                            P<int>(ctx->igrp_in), P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    else
        launch_unpack_soa(P<float>(b->in_x) + 3 * o, P<float>(b->in_v) + 3 * o, nullptr, nullptr,
                          n, P<float4>(ctx->pos_in), P<float4>(ctx->vel_in), P<int>(ctx->igrp_in),
                          P<float>(ctx->rk_in), ctx->d_err, ctx->s);
    launch_space_keys(P<float4>(ctx->pos_in), n, ctx->left, ctx->right, nullptr, 0,
                  P<uint64_t>(ctx->keys0), P<int>(ctx->vals0), ctx->s);
    build_index(ctx);
    run_knn(ctx);
    if (int r = queue_deposit(ctx, b->box[(size_t)i], b->ncs.data(), b->n_nc, b->sign, 0, nullptr, 0,
                              cap))
        return r;
    k_dens_of<<<(n + 255) / 256, 256, 0, ctx->s>>>(P<float4>(ctx->vel), n, P<float>(ctx->lab_scan));
    count_launches(1);
    launch_scatter_fields(ctx->perm, P<float>(ctx->rk), P<float>(ctx->lab_scan), nullptr, n,
                          P<float>(b->out_rk) + o, P<float>(b->out_dens) + o, nullptr, ctx->s);
    for (int k = 0; k < b->n_nc; ++k) {
        const MeshBuf& mb = ctx->meshes[(size_t)k];
        CK(cudaMemcpyAsync(P<float>(b->out_mesh) + b->mesh_off[(size_t)i * b->n_nc + k], mb.mesh.p,
                           4 * mb.words, cudaMemcpyDeviceToDevice, ctx->s));
    }
    CK(cudaMemcpyAsync(P<double>(b->out_tot) + 2 * (size_t)i * b->n_nc, ctx->totals.p,
                       16 * (size_t)b->n_nc, cudaMemcpyDeviceToDevice, ctx->s));
    return 0;
}

// eager pass over every item: sizes every buffer and records each pair count
int batch_plan(asg_batch* b)
{
    asg_ctx* ctx = b->ctx;
    const size_t S = b->sub.size();
    for (asg_ctx* c : b->sub) {
        c->leaf = ctx->leaf;  // the tuned configuration applies to every stream
        c->dep_seg = ctx->dep_seg;
        c->knn_warps = ctx->knn_warps;
        c->dep_mma = ctx->dep_mma;
        if (int r = alloc_set(c, b->max_n)) return fail(ctx, r, "batch: stream scratch");
        if (int r = grow(c, c->lab_scan, 4 * (size_t)b->max_n)) return fail(ctx, r, "batch: stream scratch");
    }
    b->cap.assign((size_t)b->n_items, 0u);
    uint32_t max_cap = 0;
    for (int i = 0; i < b->n_items; ++i) {
        asg_ctx* c = b->sub[(size_t)i % S];
        if (int r = batch_queue_item(b, c, i, 0)) return fail(ctx, r, c->last);
        const uint32_t np = c->dep_npairs;
        b->cap[(size_t)i] = np + np / 16 + 4096;  // headroom for inputs that change between runs
        max_cap = std::max(max_cap, b->cap[(size_t)i]);
    }
    for (asg_ctx* c : b->sub)
        if (int r = finish(c, "batch plan")) return fail(ctx, r, c->last);
    // reserve the deposit arrays for the largest capacity, so that the capture allocates nothing
    const size_t NP = (size_t)max_cap + 1;
    for (asg_ctx* c : b->sub) {
        int r = grow(c, c->dep_pairs, 16 * NP);
        if (!r) r = grow(c, c->dep_sort, radix_sort_temp_bytes((int)NP));
        const uint32_t items = deposit_max_items(c->dep_tiles_n, max_cap, c->dep_seg);
        if (!r) r = grow(c, c->dep_partial, deposit_partial_bytes(items) + 16);
        if (r) return fail(ctx, r, "batch: deposit reserve");
    }
    return 0;
}

int batch_capture(asg_batch* b)
{
    asg_ctx* ctx = b->ctx;
    batch_drop_graph(b);
    const size_t S = b->sub.size();
    std::vector<bool> timing;
    for (asg_ctx* c : b->sub) {
        timing.push_back(c->timing);
        c->timing = false;
    }
    const long long l0 = g_launches.load();
    cudaError_t e = cudaStreamBeginCapture(ctx->s, cudaStreamCaptureModeThreadLocal);
    int r = e == cudaSuccess ? 0 : cuda_fail(ctx, e, "cudaStreamBeginCapture");
    if (!r && S > 1) {  // fork: every stream starts after the capture origin
        if (cudaEventRecord(b->fork[0], ctx->s) != cudaSuccess) r = fail(ctx, ASG_ERR_CUDA, "fork");
        for (size_t s = 1; !r && s < S; ++s)
            if (cudaStreamWaitEvent(b->sub[s]->s, b->fork[0], 0) != cudaSuccess)
                r = fail(ctx, ASG_ERR_CUDA, "fork");
    }
    for (int i = 0; !r && i < b->n_items; ++i)
        r = batch_queue_item(b, b->sub[(size_t)i % S], i, b->cap[(size_t)i]);
    for (size_t s = 1; !r && s < S; ++s)  // join: the origin stream waits for every stream
        if (cudaEventRecord(b->join[s], b->sub[s]->s) != cudaSuccess ||
            cudaStreamWaitEvent(ctx->s, b->join[s], 0) != cudaSuccess)
            r = fail(ctx, ASG_ERR_CUDA, "join");
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) {
        const cudaError_t e2 = cudaStreamEndCapture(ctx->s, &g);
        if (!r && e2 != cudaSuccess) r = cuda_fail(ctx, e2, "cudaStreamEndCapture");
    }
    for (size_t s = 0; s < S; ++s) b->sub[s]->timing = timing[s];
    b->launches = g_launches.load() - l0;
    if (r) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return r;
    }
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) {
        batch_drop_graph(b);
        return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    return 0;
}

}  // namespace

extern "C" {

int asg_batch_create(asg_ctx* ctx, int n_items, const int* np, const int* np_local,
                     const float* left, const float* right, const float* boxsize, const int* ncs,
                     int n_nc, int sign, asg_batch** out)
{
    if (!ctx || !out || n_items <= 0 || !np || !left || !right || !boxsize || !ncs || n_nc <= 0 ||
        n_nc > MAX_MESHES)
        return fail(ctx, ASG_ERR_ARG, "bad arguments");
    *out = nullptr;
    for (int k = 0; k < n_nc; ++k)
        if (ncs[k] <= 0 || ncs[k] > 1290) return fail(ctx, ASG_ERR_ARG, "nc out of range");
    CK(cudaSetDevice(ctx->device));
    asg_batch* b = new asg_batch();
    b->ctx = ctx;
    b->n_items = n_items;
    b->n_nc = n_nc;
    b->sign = sign;
    b->ncs.assign(ncs, ncs + n_nc);
    size_t mw = 0;
    for (int i = 0; i < n_items; ++i) {
        if (np[i] < K_NN || !(left[i] < right[i]) || !(boxsize[i] > 0.0f)) {
            delete b;
            return fail(ctx, ASG_ERR_ARG, "item " + std::to_string(i) + ": bad size or bounds");
        }
        b->np.push_back(np[i]);
        b->np_local.push_back(np_local ? np_local[i] : np[i]);
        b->left.push_back(left[i]);
        b->right.push_back(right[i]);
        b->box.push_back(boxsize[i]);
        b->quant.push_back(0);
        b->cell_size.push_back(0.0f);
        b->off.push_back(b->n_total);
        b->n_total += (size_t)np[i];
        b->max_n = std::max(b->max_n, np[i]);
        for (int k = 0; k < n_nc; ++k) {
            b->mesh_off.push_back(mw);
            mw += 6 * (size_t)ncs[k] * ncs[k] * ncs[k];
        }
    }
    b->mesh_words = mw;
    int r = grow(ctx, b->in_x, 12 * b->n_total);
    if (!r) r = grow(ctx, b->in_v, 12 * b->n_total);
    if (!r) r = grow(ctx, b->out_rk, 4 * b->n_total);
    if (!r) r = grow(ctx, b->out_dens, 4 * b->n_total);
    if (!r) r = grow(ctx, b->out_mesh, 4 * mw);
    if (!r) r = grow(ctx, b->out_tot, 16 * (size_t)n_items * n_nc);
    if (!r && (cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess))
        r = fail(ctx, ASG_ERR_CUDA, "cudaEventCreate");
    b->sub.push_back(ctx);
    b->fork.assign(1, nullptr);
    b->join.assign(1, nullptr);
    if (!r && cudaEventCreateWithFlags(&b->fork[0], cudaEventDisableTiming) != cudaSuccess)
        r = fail(ctx, ASG_ERR_CUDA, "cudaEventCreate");
    if (!r) r = cudaMemsetAsync(b->in_v.p, 0, 12 * b->n_total, ctx->s) == cudaSuccess
                    ? 0 : fail(ctx, ASG_ERR_CUDA, "memset");
    if (r) {
        asg_batch_destroy(b);
        return r;
    }
    *out = b;
    return ASG_OK;
}

void asg_batch_destroy(asg_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->s);
    batch_drop_graph(b);
    for (Buf* x : {&b->in_x, &b->in_v, &b->in_cell, &b->in_off, &b->out_rk, &b->out_dens,
                   &b->out_mesh, &b->out_tot})
        if (x->p) cudaFree(x->p);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    for (size_t s = 1; s < b->sub.size(); ++s) asg_destroy(b->sub[s]);
    for (cudaEvent_t e : b->fork)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    delete b;
}

int asg_batch_set_streams(asg_batch* b, int streams)
{
    if (!b || streams < 1 || streams > 8) return ASG_ERR_ARG;
    asg_ctx* ctx = b->ctx;
    CK(cudaSetDevice(ctx->device));
    batch_drop_graph(b);
    while ((int)b->sub.size() > streams) {
        asg_destroy(b->sub.back());
        b->sub.pop_back();
        if (b->join.back()) cudaEventDestroy(b->join.back());
        b->join.pop_back();
    }
    while ((int)b->sub.size() < streams) {
        asg_ctx* c = nullptr;
        if (int r = asg_create(&c, ctx->device)) return fail(ctx, r, "batch: stream context");
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            asg_destroy(c);
            return fail(ctx, ASG_ERR_CUDA, "cudaEventCreate");
        }
        b->sub.push_back(c);
        b->join.push_back(e);
    }
    return ASG_OK;
}

int asg_batch_set_item(asg_batch* b, int item, const float* x, const float* v, int device_ptrs)
{
    if (!b || !x || item < 0 || item >= b->n_items) return ASG_ERR_ARG;
    asg_ctx* ctx = b->ctx;
    CK(cudaSetDevice(ctx->device));
    if (b->quant[(size_t)item] != 0) batch_drop_graph(b);  // the item's unpack kernel changes
    b->quant[(size_t)item] = 0;
    const size_t o = b->off[(size_t)item], bytes = 12 * (size_t)b->np[(size_t)item];
    const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CK(cudaMemcpyAsync(P<float>(b->in_x) + 3 * o, x, bytes, kind, ctx->s));
    if (v) CK(cudaMemcpyAsync(P<float>(b->in_v) + 3 * o, v, bytes, kind, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ASG_OK;
}

int asg_batch_set_item_quantised(asg_batch* b, int item, const int* cell, const uint16_t* off,
                                 const float* v, float cell_size, int grid, int device_ptrs)
{
    if (!b || !cell || !off || item < 0 || item >= b->n_items) return ASG_ERR_ARG;
    asg_ctx* ctx = b->ctx;
    const size_t i = (size_t)item;
    if (int r = check_quant(ctx, grid, cell_size, b->left[i], b->right[i])) return r;
    CK(cudaSetDevice(ctx->device));
    if (int r = grow(ctx, b->in_cell, 4 * b->n_total)) return r;
    if (int r = grow(ctx, b->in_off, 6 * b->n_total)) return r;
    if (b->quant[i] != grid || b->cell_size[i] != cell_size) batch_drop_graph(b);
    b->quant[i] = grid;
    b->cell_size[i] = cell_size;
    const size_t o = b->off[i], np = (size_t)b->np[i];
    const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CK(cudaMemcpyAsync(P<int>(b->in_cell) + o, cell, 4 * np, kind, ctx->s));
    CK(cudaMemcpyAsync(P<uint16_t>(b->in_off) + 3 * o, off, 6 * np, kind, ctx->s));
    if (v) CK(cudaMemcpyAsync(P<float>(b->in_v) + 3 * o, v, 12 * np, kind, ctx->s));
    else CK(cudaMemsetAsync(P<float>(b->in_v) + 3 * o, 0, 12 * np, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ASG_OK;
}

int asg_batch_tune(asg_batch* b, int* leaf, int* seg)
{
    if (!b) return ASG_ERR_ARG;
    asg_ctx* ctx = b->ctx;
    CK(cudaSetDevice(ctx->device));
    if (int r = alloc_set(ctx, b->max_n)) return r;
    if (int r = grow(ctx, ctx->lab_scan, 4 * (size_t)b->max_n)) return r;
    int item = 0;  // the largest item
    for (int i = 1; i < b->n_items; ++i)
        if (b->np[(size_t)i] > b->np[(size_t)item]) item = i;
    // tree bucket size x deposit work-item length x neighbour-search warps per
    // block x deposit engine (tensor cores or CUDA cores)
    const int leaves[] = {16, 24, 32}, segs[] = {2048, 4096, 8192}, warps[] = {2, 4}, mmas[] = {1, 2, 0};
    float best = INFINITY;
    int bl = ctx->leaf, bs = ctx->dep_seg, bw = ctx->knn_warps, bm = ctx->dep_mma;
    for (int l : leaves)
        for (int sg : segs)
            for (int w : warps)
                for (int m : mmas) {
                    ctx->leaf = l;
                    ctx->dep_seg = sg;
                    ctx->knn_warps = w;
                    ctx->dep_mma = m;
                    float ms = 0.0f;
                    for (int rep = 0; rep < 2; ++rep) {  // the first repetition warms up
                        CK(cudaEventRecord(b->e0, ctx->s));
                        if (int r = batch_queue_item(b, ctx, item, 0)) return r;
                        CK(cudaEventRecord(b->e1, ctx->s));
                        CK(cudaEventSynchronize(b->e1));
                        CK(cudaEventElapsedTime(&ms, b->e0, b->e1));
                    }
                    if (ms < best) {
                        best = ms;
                        bl = l;
                        bs = sg;
                        bw = w;
                        bm = m;
                    }
                }
    ctx->leaf = bl;
    ctx->dep_seg = bs;
    ctx->knn_warps = bw;
    ctx->dep_mma = bm;
    batch_drop_graph(b);  // a new configuration needs a new plan and capture
    if (leaf) *leaf = bl;
    if (seg) *seg = bs;
    return finish(ctx, "batch tune");
}

int asg_batch_config(asg_batch* b, int* leaf, int* seg, int* knn_warps, int* deposit_engine)
{
    if (!b) return ASG_ERR_ARG;
    const asg_ctx* ctx = b->ctx;
    if (leaf) *leaf = ctx->leaf;
    if (seg) *seg = ctx->dep_seg;
    if (knn_warps) *knn_warps = ctx->knn_warps;
    if (deposit_engine) *deposit_engine = ctx->dep_mma;
    return ASG_OK;
}

int asg_batch_run(asg_batch* b)
{
    if (!b) return ASG_ERR_ARG;
    asg_ctx* ctx = b->ctx;
    CK(cudaSetDevice(ctx->device));
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (!b->exec) {
            if (int r = batch_plan(b)) return r;
            if (int r = batch_capture(b)) return r;
        }
        CK(cudaEventRecord(b->e0, ctx->s));
        CK(cudaGraphLaunch(b->exec, ctx->s));
        CK(cudaEventRecord(b->e1, ctx->s));
        count_launches((int)b->launches);
        int r = finish(ctx, "batch run");
        for (size_t s = 1; s < b->sub.size(); ++s) {  // the other streams' error words
            const int rs = finish(b->sub[s], "batch run");
            if (rs && (!r || r == ASG_ERR_STATE)) r = fail(ctx, rs, b->sub[s]->last);
        }
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, b->e0, b->e1) == cudaSuccess) b->last_ms = ms;
        if (r != ASG_ERR_STATE) return r;  // ERR_CAP: the inputs outgrew the plan
        batch_drop_graph(b);
    }
    return fail(ctx, ASG_ERR_STATE, "batch: pair capacity exceeded twice");
}

int asg_batch_stats(asg_batch* b, double* graph_ms, long long* kernels, long long* particles_local)
{
    if (!b) return ASG_ERR_ARG;
    if (graph_ms) *graph_ms = b->last_ms;
    if (kernels) *kernels = b->launches;
    if (particles_local) {
        long long s = 0;
        for (int v : b->np_local) s += v;
        *particles_local = s;
    }
    return ASG_OK;
}

int asg_batch_get(asg_batch* b, int item, float* rk, float* dens, float* const* meshes,
                  double* totals)
{
    if (!b || item < 0 || item >= b->n_items) return ASG_ERR_ARG;
    asg_ctx* ctx = b->ctx;
    CK(cudaSetDevice(ctx->device));
    const size_t o = b->off[(size_t)item], n = (size_t)b->np[(size_t)item];
    if (rk) CK(cudaMemcpyAsync(rk, P<float>(b->out_rk) + o, 4 * n, cudaMemcpyDeviceToHost, ctx->s));
    if (dens) CK(cudaMemcpyAsync(dens, P<float>(b->out_dens) + o, 4 * n, cudaMemcpyDeviceToHost, ctx->s));
    for (int k = 0; meshes && k < b->n_nc; ++k)
        if (meshes[k]) {
            const size_t nc = (size_t)b->ncs[(size_t)k];
            CK(cudaMemcpyAsync(meshes[k], P<float>(b->out_mesh) + b->mesh_off[(size_t)item * b->n_nc + k],
                               24 * nc * nc * nc, cudaMemcpyDeviceToHost, ctx->s));
        }
    if (totals)
        CK(cudaMemcpyAsync(totals, P<double>(b->out_tot) + 2 * (size_t)item * b->n_nc,
                           16 * (size_t)b->n_nc, cudaMemcpyDeviceToHost, ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
    return ASG_OK;
}

}  // extern "C"
