// asg_internal.h -- device data layout and kernel launchers shared by the
// translation units of libasmooth_gb300.so (not part of the public C ABI).
//
// Data layout in HBM (one particle set, N particles):
//   pos   float4[N]  x, y, z, w = input index (int bits)   -- Hilbert order
//   vel   float4[N]  vx, vy, vz, dens                        -- Hilbert order
//   igrp  int[N]                                             -- Hilbert order
//   rk    float[N], t33 float[N], idx33 int[N]               -- Hilbert order
// Radix tree over the N sorted space-filling-curve keys (Karras 2012), N-1 internal nodes:
//   meta  int4[N-1]  child0, child1 (>=0 internal, <0 leaf ~i), first, last
//   blo/bhi float4[N-1]  AABB of the node's particles
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace asg {

// process-wide count of kernel launches made by this library
void count_launches(int k);

struct TreeView {
    int n;                 // particles (leaves)
    int leaf;              // bucket size: nodes with <= leaf particles are scanned whole (1..32)
    const int4* meta;      // internal nodes 0..n-2 (root 0); empty when n == 1
    const float4* blo;
    const float4* bhi;
    // 64 bytes per internal node, one load round trip per visit: word 0 the
    // meta (c0, c1, first, last as int bits); words 1-3 the boxes of both
    // children of a node with more than `leaf` particles (a leaf child as its
    // point: lo0.xyz hi0.x | hi0.yz lo1.xy | lo1.z hi1.xyz), or the node's own
    // box for a bucket (lo.xyz hi.x | hi.yz)
    const float4* rec;
};

// root entry of a traversal: internal node 0, or leaf 0 when n == 1
__host__ __device__ inline int tree_root(int n) { return n > 1 ? 0 : ~0; }

// ---- index build (asg_index.cu) -------------------------------------------------
// unpack reference Particle records (36 B), or SoA device arrays, into the
// staging arrays (input order; pos.w carries the input index)
void launch_unpack_aos(const void* aos, int n, float4* pos_in, float4* vel_in, int* igrp_in,
                       float* rk_in, int* err, cudaStream_t s);
void launch_unpack_soa(const float* x, const float* v, const float* dens, const int* igrp, int n,
                       float4* pos_in, float4* vel_in, int* igrp_in, float* rk_in, int* err,
                       cudaStream_t s);
// mixed-precision positions: int32 cell index + 3 x uint16 offsets in cells of side cs
void launch_unpack_quant(const int* cell, const uint16_t* off, const float* v, int n, int grid,
                         float left, float cs, float4* pos_in, float4* vel_in, int* igrp_in,
                         float* rk_in, int* err, cudaStream_t s);
// 48-bit Hilbert keys (16 bits per axis; Morton with ASG_SPACE_CURVE=morton)
// over [left, right)^3, or over the particles' own bounding cube when d_lohi
// (2 ints of scratch) is given; key_prefix lands in bits 48+ (batched cubes)
void launch_space_keys(const float4* pos_in, int n, float left, float right, int* d_lohi,
                       uint64_t key_prefix, uint64_t* keys, int* vals, cudaStream_t s);
// stable LSD radix sort of (keys, vals) on the low `bits` bits; ping-pong buffers;
// returns which buffer (0/1) holds the result
size_t radix_sort_temp_bytes(int n);
int radix_sort32(uint32_t* keys0, int* vals0, uint32_t* keys1, int* vals1, int n, int bits,
                 void* temp, cudaStream_t s);
int radix_sort(uint64_t* keys0, int* vals0, uint64_t* keys1, int* vals1, int n, int bits,
               void* temp, cudaStream_t s);
void launch_gather_sorted(const int* perm, const float4* pos_in, const float4* vel_in,
                          const int* igrp_in, const float* rk_in, int n, float4* pos, float4* vel,
                          int* igrp, float* rk, cudaStream_t s);
void launch_iota(int* a, int n, cudaStream_t s);
// err |= ERR_ZERO_RK when some rk is not a positive finite number
void launch_check_rk(const float* rk, int n, int* err, cudaStream_t s);
void launch_build_tree(const uint64_t* keys, int n, int4* meta, int* parent, int* leaf_parent,
                       cudaStream_t s);
// bottom-up AABBs of the nodes a traversal with bucket size `leaf` reads (the
// root and the children of nodes with more than leaf particles); with
// rk != nullptr the expanded boxes [x-h', x+h']; rec (or null) receives
// TreeView::rec of those nodes (4 float4 per internal node)
void launch_tree_boxes(const float4* pos, const float* rk, int n, int leaf, const int4* meta,
                       const int* parent, int* flags, float4* lo, float4* hi, float4* rec,
                       cudaStream_t s);
// exclusive scan of uint32 counts (in place); temp from scan_temp_bytes
size_t scan_temp_bytes(size_t n);
void exclusive_scan_u32(uint32_t* data, size_t n, void* temp, cudaStream_t s);

// ---- neighbour search (asg_knn.cu) -------------------------------------------
// Buckets k_knn_t33 scanned, per 32-query bundle: word 0 = their count (-1 when
// more than KNN_LIST), then the node ids (a bucket node, or ~i for one particle).
// k_dens_scatter visits these instead of walking the tree again.
constexpr int KNN_LIST = 96;
inline size_t knn_list_words(int n) { return (size_t)((n + 31) / 32) * (KNN_LIST + 1); }
// t33, rk = sqrtf(t33), idx33 = -1 (no tie at the 33rd) or -2 (ties to resolve);
// blist (knn_list_words ints, or null) receives the scanned buckets; warps: 2 or
// 4 warps per block (tuning)
void launch_knn_t33(const float4* pos, const TreeView& t, float* t33, float* rk, int* idx33,
                    int* blist, int* err, cudaStream_t s, int warps = 2);
// idx33 = input index of the 33rd key, for flagged queries (all = 0) or every query
void launch_knn_ties(const float4* pos, const TreeView& t, const float* t33, int* idx33,
                     int all, int* err, cudaStream_t s);
// vel[j].w (dens) += the tent weights j receives as one of the 32 nearest;
// dexp (n ints) and acc (n uint64) are scratch; blist from launch_knn_t33 or null
void launch_dens(const float4* pos, const TreeView& t, const float* t33, const int* idx33,
                 const int* blist, const float* rk, int* dexp, unsigned long long* acc,
                 float4* vel, int* err, cudaStream_t s);

// ---- mesh deposit (asg_deposit.cu) ---------------------------------------------
struct MeshJob {
    int nc;           // cells per dimension
    float dx;         // boxsize / nc (host float division, as the reference)
    float ncf;        // (float)nc
    int tiles[3];     // tiles per dimension
    int tile_begin;   // first global tile id of this mesh
    float* mesh;      // 6*nc^3 floats (reference layout) or nc^3 (density only)
    double* partial;  // per-tile FP64 partial sums, 2 per tile (n, halo)
};
constexpr int MAX_MESHES = 8;
struct DepositParams {
    int n_jobs;
    MeshJob job[MAX_MESHES];
    float boxsize;
    float rbox;       // 1/boxsize rounded to nearest (for div_rn_by)
    int sign;
    int periodic;
    float offset[3];  // periodic: rank cube offset
    int density_only;
    int seg;          // pairs per work item of the persistent deposit (tuning, > 0)
    int mma;          // the deposit engine: 1 or 2 tensor cores (one or two warps per
                      // item), 0 the CUDA cores (tuning)
    // the order in which the persistent deposit takes the tiles (slot -> tile)
    // and its inverse (tile -> slot), or null for tile order: tiles of every
    // mesh sorted by position along a Morton curve, coarse before fine at the
    // same place, so that the tiles of all meshes that read the same particle
    // records run close together in time and find them in L2
    const uint32_t* order;
    const uint32_t* pos;
};
// the processing order above for the meshes of p (host; 2 * total tiles words:
// order, then pos)
void deposit_tile_order(const DepositParams& p, int total_tiles, uint32_t* out);
// scratch of one deposit: particle records, (tile, image) pairs, work items
struct DepositScratch {
    float4* rec;          // [2n] x', y', z', h (-h: halo channel, 0: skipped) | dens, v
    uint32_t* pcount;     // [n+1] pairs per particle, then their exclusive scan
    void* scan_tmp_n;     // scan scratch for n+1 entries
    uint32_t* keys0;      // [npairs] tile << 5 | image (periodic), else tile; ping-pong with keys1
    uint32_t* keys1;
    int* vals0;           // [npairs] particle (sorted position), ping-pong with vals1
    int* vals1;
    void* sort_tmp;       // radix sort scratch for npairs
    uint32_t* tstart;     // [T] first pair of each tile
    uint32_t* tcount;     // [T] pairs of each tile
    uint32_t* item_off;   // [T+1] exclusive scan of work items per tile
    void* scan_tmp_t;     // scan scratch for T+1 entries
    float* partial;       // [items] partial tiles of multi-segment tiles
    int* next_item;       // work counter of the persistent kernel
};
size_t deposit_prep_bytes(int n);
size_t deposit_tile_bytes(int total_tiles);
uint32_t deposit_max_items(int total_tiles, uint32_t npairs, int seg);
int deposit_default_seg();
int deposit_default_mma();
size_t deposit_partial_bytes(uint32_t items);
// pass 1: particle records and pair counts; pcount[n] then holds the number of pairs
void launch_deposit_prep(const float4* pos, const float4* vel, const int* igrp, const float* rk,
                         int n, const DepositParams& p, DepositScratch& w, int* err,
                         cudaStream_t s);
// pass 2: emit and sort the pairs, deposit every (tile, segment), merge multi-segment tiles.
// padded = false: npairs is the exact pair count (read back from pcount[n]);
// padded = true: npairs is the arrays' capacity, the count stays on the device
// (no host synchronisation, e.g. under stream capture) and a larger count sets ERR_CAP
void launch_deposit_run(int n, const DepositParams& p, int total_tiles, uint32_t npairs, bool padded,
                        DepositScratch& w, int* err, cudaStream_t s);
void launch_reduce_partials(const double* partial, int ntiles, double* out2, cudaStream_t s);
void launch_normalise(float* mesh, int nc, float vol, cudaStream_t s);

// ---- FOF and SO halos (asg_fof.cu) -----------------------------------------------
void launch_fof_link(const float4* pos, const TreeView& t, float ll, int* parent, int* err,
                     cudaStream_t s);
void launch_fof_finish(const float4* pos, int n, int* parent, int* minin, int* mark,
                       cudaStream_t s);
void launch_fof_label(const float4* pos, int n, const int* parent, const int* minin,
                      const uint32_t* scan, int* igrp_sorted, cudaStream_t s);
void launch_mark_halos(const float4* pos, const TreeView& t, const float* halos, int nh,
                       float left, float right, int* igrp, long long* counts, double* mass8,
                       cudaStream_t s);
void launch_count_labels(const int* igrp, int n, uint32_t* counts, cudaStream_t s);
void launch_keep_mask(uint32_t* counts, int ngrp, int threshold, cudaStream_t s);
void launch_relabel(int* igrp, int n, const uint32_t* scan, const uint32_t* keep, cudaStream_t s);

// ---- periodic buffer shell of a single-cube run (asg_shell.cu) ------------------------------
// base[b][d]: first slot of the copies of bin b sent in direction d (-1: none)
struct ShellPlan {
    int base[27][27];
};
void launch_shell_bins(const float4* pos, int n, float lt, float rt, uint32_t* keys0, int* vals0,
                       uint32_t* keys1, int* vals1, void* sort_tmp, uint32_t* start, uint32_t* end,
                       const uint32_t** keys, const int** order, cudaStream_t s);
void launch_shell_emit(const float4* pos, const float4* vel, const int* igrp, const float* rk,
                       const uint32_t* keys, const int* order, const uint32_t* start, int n,
                       const ShellPlan& plan, float L, float4* apos, float4* avel, int* aigrp,
                       float* ark, cudaStream_t s);
// keep -bf*L < x < L + bf*L; flags has n_all + 1 words and ends as the exclusive scan
void launch_shell_filter(const float4* apos, const float4* avel, const int* aigrp, const float* ark,
                         int n_all, float lo, float hi, uint32_t* flags, void* scan_tmp,
                         float4* pos, float4* vel, int* igrp, float* rk, cudaStream_t s);

// ---- particle file payloads (asg_decode.cu) ----------------------------------------------
void launch_decode_xv(const float* xv, int n, const float* shift, float4* pos, float4* vel,
                      int* igrp, float* rk, int* err, cudaStream_t s);
size_t zip_scratch_bytes(int ncell);
// *start: first particle of every cell, ncell + 1 entries (the last = total)
void launch_zip_counts(const uint8_t* c8, const int* c32, int n32, int ncell, void* scratch,
                       uint32_t** start, int* err, cudaStream_t s);
void launch_zip_particles(const uint8_t* off, const int16_t* vq, const uint32_t* start, int ncell,
                          int nc, int n, int mesh_scale, float v_r2i, const float* shift,
                          float4* pos, float4* vel, int* igrp, float* rk, cudaStream_t s);

// ---- FOF halo catalogue and file formats (asg_output.cu) ----------------------------------
// records {x[3], v[3], int nfof} of labels 1..nhalo with centre inside (0, boxsize)^3, label
// order, into out (device, 7*nhalo words) and *nlocal (device); pos/vel/igrp indexed by j,
// the caller's array index is pos[j].w when w_index else j
size_t fof_catalogue_bytes(int n, int nhalo);
void launch_fof_catalogue(const float4* pos, const float4* vel, const int* igrp, int n, int w_index,
                          int nhalo, float boxsize, void* scratch, float* out, uint32_t* nlocal,
                          cudaStream_t s);
int write_mesh_files(const char* base, int inode, const float* mesh, int nc);
int write_fof_file(const char* filename, const float* rec, int nlocal);

// ---- output (asg_index.cu) ------------------------------------------------------------
// write reference Particle records in input order from the sorted fields
void launch_pack_aos(const int* perm, const float4* pos, const float4* vel, const float* rk,
                     const float* dens, const int* igrp, int n, void* aos, cudaStream_t s);
void launch_scatter_fields(const int* perm, const float* rk, const float* dens, const int* igrp,
                           int n, float* rk_out, float* dens_out, int* igrp_out, cudaStream_t s);

}  // namespace asg
