/*
 * asmooth_gb300.h -- C ABI of the GB300 adaptive-smoothing path.
 *
 * Drop-in replacement for the hot path of junkoda/asmooth's clumping_tree:
 * kd-tree construction, the k=32 (+self) neighbour search with smoothing length
 * and particle density, the adaptive mesh deposit at several nc, the FP64 mass
 * totals, the output normalisation, friends-of-friends and SO-halo marking.
 * The host keeps every buffer; the library owns device memory and one CUDA
 * stream per context.  All calls are synchronous at return, return an int
 * status (0 = ASG_OK) and never throw.  One context per host thread; a
 * context is not thread-safe.
 *
 * Particle records are the reference's `struct Particle` (basic_types.h:10-15),
 * 36 bytes: float x[3], v[3], dens, rk; int igrp.  Halo records are the
 * reference's `struct Halo` (basic_types.h:17-20): float x[3], r, mass.
 * Unlike the reference, no call reorders the caller's particle array.
 */
#ifndef ASMOOTH_GB300_H
#define ASMOOTH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASG_ABI_VERSION 2

typedef struct asg_particle {
    float x[3], v[3];
    float dens, rk;
    int igrp;
} asg_particle;

typedef struct asg_halo {
    float x[3];
    float r, mass;
} asg_halo;

typedef struct asg_ctx asg_ctx;

enum {
    ASG_OK = 0,
    ASG_ERR_ARG = -1,         /* bad argument (null pointer, n or nc out of range) */
    ASG_ERR_CUDA = -2,        /* CUDA runtime error (see asg_last_error) */
    ASG_ERR_NOMEM = -3,       /* device allocation failed */
    ASG_ERR_FEW = -4,         /* fewer than 33 particles can be reached by a query */
    ASG_ERR_ZERO_RK = -5,     /* 33rd neighbour distance is 0 (>= 33 coincident particles) */
    ASG_ERR_NONFINITE = -6,   /* NaN or infinite position */
    ASG_ERR_STACK = -7,       /* tree deeper than the traversal stack */
    ASG_ERR_TIES = -8,        /* more than 16 particles tied exactly at the 33rd distance */
    ASG_ERR_RANGE = -9,       /* periodic deposit: kernel support wider than the mesh */
    ASG_ERR_STATE = -10,      /* call needs a previous step (e.g. deposit before search) */
    ASG_ERR_UNIONFIND = -11,  /* FOF union-find retry limit reached */
    ASG_ERR_NOALLOC_LIMIT = -12, /* input larger than the allocation-free entry point's fixed scratch */
    ASG_ERR_IO = -13            /* an output file could not be opened or written */
};

/* ---- context ------------------------------------------------------------- */
int asg_create(asg_ctx** ctx, int device);
void asg_destroy(asg_ctx* ctx);
const char* asg_strerror(int status);
/* text of the last error seen by this context (CUDA message or argument check) */
const char* asg_last_error(asg_ctx* ctx);
int asg_abi_version(void);

/* ---- host memory for particle and mesh arrays --------------------------------
 * Page-locked host memory that the copies in asg_smooth and the other
 * host-array calls read and write at the link's rate on every call.  Blocks of
 * at least half a transparent huge page are whole huge pages, mapped on
 * huge-page boundaries and advised as huge pages before CUDA pins them
 * (registered portable, usable from every device); smaller blocks are pinned
 * base pages, so several small arrays are best carved from one block.  On the
 * Grace hosts of GB300 nodes (64 KB base pages, 512 MB huge pages) some copies
 * of hundreds of MB from ordinary pinned memory ran at 10-30 GB/s instead of
 * about 200; from huge-page blocks they did not.  *out is null on failure.
 * Free with asg_host_free (null is a no-op; a pointer this call did not
 * return is ASG_ERR_ARG). */
int asg_host_alloc(size_t bytes, void** out);
int asg_host_free(void* p);

/* ---- reference-shaped one-shot calls (host arrays) --------------------------- */

/* Tree construction + neighbour search for every particle
 * (replaces clumping_tree_main.cpp:390-395 and :418-430 around
 * KDTree::construct, kdtree_balanced.h:17, and neighbor_search,
 * nbr_search.h:9).  Sets p[i].rk = sqrtf(d2 of the 33rd nearest, self
 * included) and adds to p[i].dens the tent weights of every query that has i
 * among its 32 nearest.  Neighbours are the 33 smallest keys (d2, index).
 * [left, right) is the buffered cube (-b*L, (1+b)*L). */
int asg_neighbor_search(asg_ctx* ctx, asg_particle* p, int np, float left, float right);

/* clear_mesh + assign_on_mesh for one mesh (coarse_mesh.h:4-8, called at
 * clumping_tree_main.cpp:525-526): mesh gets 6*nc^3 floats in the reference
 * layout [n | halo | c | v (xyz interleaved)].  totals (optional, 2 doubles):
 * FP64 sums of the n and halo weights (mesh_total, coarse_mesh.h:5). */
int asg_assign_on_mesh(asg_ctx* ctx, const asg_particle* p, int np, float boxsize, int nc,
                       int sign, float* mesh, double* totals);

/* The whole per-nc loop (clumping_tree_main.cpp:521-533) in one call:
 * meshes[k] receives mesh k (6*ncs[k]^3 floats), totals[2k..2k+1] its FP64
 * Σn, Σhalo.  periodic=1 is assign_on_global_mesh (global_mesh.cpp:25-28) for
 * the rank at grid coordinates coords[3] (offset = boxsize*coords). */
int asg_assign_on_meshes(asg_ctx* ctx, const asg_particle* p, int np, float boxsize,
                         const int* ncs, int n_nc, int sign, int periodic, const int* coords,
                         float* const* meshes, double* totals);

/* assign_on_density_mesh (coarse_mesh.h:14-16): n channel only, nc^3 floats. */
int asg_assign_on_density_mesh(asg_ctx* ctx, const asg_particle* p, int np, float boxsize,
                               int nc, int sign, float* mesh);

/* write_mesh_separate normalisation (coarse_mesh.cpp:158-171) of a host mesh,
 * in place: c *= vol/n^2, v /= n, n *= 8, halo *= 8 (vol = powf(L/nc, 3)). */
int asg_normalise_mesh(asg_ctx* ctx, float* mesh, int nc, float boxsize);

/* group_fof (fof.h:7-9, called at clumping_tree_main.cpp:405): p[i].igrp gets
 * group labels 1..ngroup (every particle is in a group), numbered in order of
 * each group's smallest input index.  ll is the internal linking length. */
int asg_group_fof(asg_ctx* ctx, asg_particle* p, int np, float left, float right, float ll,
                  int* ngroup);

/* remove_small_groups (fof.h:11-12): groups with >= 20 members -> 1..nhalo in
 * label order, all others -> 0.  Labels must be in [0, ngrp]. */
int asg_remove_small_groups(asg_ctx* ctx, asg_particle* p, int np, int ngrp, int* nhalo);

/* The SO-halo loop at clumping_tree_main.cpp:465-485 around
 * mark_halo_particles (nbr_search.h:11): for every halo whose centre is
 * strictly inside (left, right)^3, particles with d2 < r*r get igrp = -1;
 * np_halo = sum of the per-halo counts, m_halo = sum of mass/8. */
int asg_mark_halo_particles(asg_ctx* ctx, asg_particle* p, int np, const asg_halo* halos,
                            int nh, float left, float right, long* np_halo, double* m_halo);

/* The per-redshift hot path in one call: tree, neighbour search, SO-halo
 * marking (nh may be 0), then the deposit for every nc with sign, written to
 * meshes[k] (host, 6*nc^3 floats each) and totals[2k..2k+1].  p is updated in
 * place (rk, dens, igrp). */
int asg_smooth(asg_ctx* ctx, asg_particle* p, int np, float left, float right, float boxsize,
               const asg_halo* halos, int nh, const int* ncs, int n_nc, int sign,
               float* const* meshes, double* totals, long* np_halo, double* m_halo);

/* ---- outputs ------------------------------------------------------------------ */

/* write_mesh_separate (coarse_mesh.cpp:147-208, called at
 * clumping_tree_main.cpp:446-447 and :531-532): normalises the host mesh in
 * place (as asg_normalise_mesh) and writes <base>n<inode>.dat,
 * <base>h<inode>.dat, <base>c<inode>.dat (int nc, nc^3 floats each) and
 * <base>vel<inode>.dat (int nc, 3*nc^3 floats), byte for byte the reference's
 * files.  The directories must exist.  ASG_ERR_IO when a file fails. */
int asg_write_mesh_separate(asg_ctx* ctx, const char* base, int inode, float* mesh, int nc,
                            float boxsize);
/* The same for device mesh k of the last asg_run_deposit (normalised in place). */
int asg_write_mesh_device(asg_ctx* ctx, int k, const char* base, int inode);
/* write_mesh (coarse_mesh.cpp:128-143): int nc, int 6, float boxsize, then the
 * 6*nc^3 floats of the mesh as they are.  Host only. */
int asg_write_mesh(const char* filename, const float* mesh, int nc, float boxsize);

/* struct FofHalo (fof.cpp:22-25), 28 bytes */
typedef struct asg_fof_halo {
    float x[3], v[3];
    int nfof;
} asg_fof_halo;

/* The catalogue of write_fof_halos (fof.cpp:169-219) for labels 1..nhalo (the
 * output of asg_remove_small_groups): per halo the float sums of x and v over
 * its members in array order divided by the member count; halos whose centre
 * is strictly inside (0, boxsize)^3 go to out[0..*nlocal-1] in label order
 * (out holds nhalo records).  Same bits as the reference on the same array,
 * except that v[2] starts from 0 (the reference never clears it, fof.cpp:179). */
int asg_fof_halos(asg_ctx* ctx, const asg_particle* p, int np, int nhalo, float boxsize,
                  asg_fof_halo* out, int* nlocal);
/* write_fof_halos' file: int nlocal, int 28, the records, int nlocal. */
int asg_write_fof_halos(asg_ctx* ctx, const char* filename, const asg_particle* p, int np,
                        int nhalo, float boxsize);

/* ---- staged device-resident interface --------------------------------------- */

/* Load a particle set and build its index (H2D + sort + tree).  Subsequent
 * asg_run_* calls work on it until the next load. */
int asg_load_particles(asg_ctx* ctx, const asg_particle* p, int np, float left, float right);
/* Same from device arrays: x (np*3), v (np*3, may be NULL), dens (np, may be
 * NULL = 0), igrp (np, may be NULL = 0). */
int asg_load_particles_device(asg_ctx* ctx, const float* d_x, const float* d_v,
                              const float* d_dens, const int* d_igrp, int np, float left,
                              float right);
/* Single-cube periodic run: the np_local particles of the whole box [0, L)^3
 * plus the buffer shell built on the device, replacing the one-rank
 * exchange_buffer (exchange_buffer.cpp:13-168, every direction a
 * self-exchange with x -= (d-1)*L) and remove_extra_particles
 * (clumping_tree_main.cpp:550-576, keep -bf*L < x < L + bf*L), then the index
 * build as asg_load_particles with left = -bf*L, right = L + bf*L.  The same
 * particles and float positions as the reference; order: the np_local
 * particles as given, then the copies grouped by (source bin, direction) in
 * the reference's loop order, each group in input order (the reference orders
 * a bin by an in-place swap sort).  *np_with_buffers receives the set size
 * (read it back with asg_store_particles into that many records),
 * *np_local_kept the interior particles kept. */
int asg_load_periodic_cube(asg_ctx* ctx, const asg_particle* p, int np_local, float boxsize,
                           float buffer_factor, int* np_with_buffers, int* np_local_kept);
int asg_load_periodic_cube_device(asg_ctx* ctx, const float* d_x, const float* d_v, int np_local,
                                  float boxsize, float buffer_factor, int* np_with_buffers,
                                  int* np_local_kept);

/* ---- particle files decoded on the device ------------------------------------
 * The conversion of read_pm_file_xv (file_reader2.cpp:24-86: x - shift, v,
 * rk = dens = igrp = 0) and the count-prefix expansion of read_pm_file_zip
 * (file_reader2.cpp:90-272: x = mesh_scale*((off + 0.5f)/256.0f + i - 1.0f)
 * - shift in that float order, v = vel / v_r2i; little-endian files) run on
 * the device; the decoded particles stay there for asg_load_decoded_periodic
 * and can be read back with asg_copy_decoded. */
/* xv: np records of 6 floats (x, y, z, vx, vy, vz), the payload after the 48-byte header. */
int asg_decode_xv(asg_ctx* ctx, const float* xv, int np, const float* shift);
/* zip: zip0 payload (3*np_local offsets), zip1 payload (3*np_local int16), zip2
 * (nc_node_dim^3 counts), zip3 (n_zip3 int32 counts of the cells marked 255).
 * ASG_ERR_ARG when the counts do not sum to np_local (the reference's
 * ErrorParticleReader) or a 255-cell has no zip3 entry. */
int asg_decode_zip(asg_ctx* ctx, const uint8_t* zip0, const int16_t* zip1, const uint8_t* zip2,
                   const int* zip3, int n_zip3, int np_local, int nc_node_dim, int mesh_scale,
                   float v_r2i, const float* shift);
/* read_pm_file_xv / read_pm_file_zip (file_reader2.h): read
 * <filebase><inode>/<redshift>xv<inode>.dat or <redshift>zip{0..3}_<inode>.dat
 * on the host and decode on the device; *np = np_local, *boxsize = mesh_scale *
 * nc_node_dim (zip).  ASG_ERR_IO when a file cannot be read, ASG_ERR_ARG when
 * sizes disagree (the reference asserts). */
int asg_read_pm_file_xv(asg_ctx* ctx, const char* filebase, const char* redshift, int inode,
                        const float* shift, int* np);
int asg_read_pm_file_zip(asg_ctx* ctx, const char* filebase, const char* redshift, int inode,
                         int nc_node_dim, int mesh_scale, const float* shift, int* np,
                         float* boxsize);
/* The decoded particles as Particle records (np of them, in file order). */
int asg_copy_decoded(asg_ctx* ctx, asg_particle* out);
/* asg_load_periodic_cube on the decoded particles, without a host round trip. */
int asg_load_decoded_periodic(asg_ctx* ctx, float boxsize, float buffer_factor,
                              int* np_with_buffers, int* np_local_kept);

int asg_run_neighbor_search(asg_ctx* ctx);
int asg_run_mark_halos(asg_ctx* ctx, const asg_halo* halos, int nh, long* np_halo,
                       double* m_halo);
int asg_run_fof(asg_ctx* ctx, float ll, int* ngroup);
int asg_run_remove_small_groups(asg_ctx* ctx, int ngrp, int* nhalo);
/* Catalogue of the loaded set's labels (as asg_fof_halos), array order = load order. */
int asg_run_fof_halos(asg_ctx* ctx, int nhalo, float boxsize, asg_fof_halo* out, int* nlocal);
/* Deposit for every nc into library-owned device meshes (read them with
 * asg_mesh_device or asg_copy_mesh); totals (host, 2 per mesh) optional. */
int asg_run_deposit(asg_ctx* ctx, float boxsize, const int* ncs, int n_nc, int sign,
                    int periodic, const int* coords, int density_only, double* totals);
/* Normalise device mesh k in place (write_mesh_separate semantics). */
int asg_run_normalise(asg_ctx* ctx, int k);
/* Device pointer of mesh k from the last asg_run_deposit. */
float* asg_mesh_device(asg_ctx* ctx, int k);
int asg_copy_mesh(asg_ctx* ctx, int k, float* host);
/* Write the loaded set back (input order) as Particle records. */
int asg_store_particles(asg_ctx* ctx, asg_particle* p);
/* Input-order fields to device arrays (any may be NULL). */
int asg_store_fields_device(asg_ctx* ctx, float* d_rk, float* d_dens, int* d_igrp);
/* Neighbour-search internals in input order (host arrays, any may be NULL):
 * t33 = d2 of the 33rd key, idx33 = its input index. */
int asg_get_knn(asg_ctx* ctx, float* t33, int* idx33);

/* ---- mixed-precision form ---------------------------------------------------------
 * No counterpart in the reference, whose positions are always float x[3]:
 * positions arrive as one int32 cell index c = (cz*grid + cy)*grid + cx of a
 * cubic grid of side cell_size starting at left, plus three uint16 offsets
 * (np*3, xyz interleaved) in units of cell_size/65536.  The device decodes
 *   x = (left + cell_size*cx) + off_x*(cell_size/65536)
 * with every product and sum rounded to nearest float in this order, then runs
 * the same FP32 path as the plain form, so the results equal the plain form's
 * on the decoded positions.  grid*cell_size must cover [left, right); a cell
 * index outside [0, grid^3) returns ASG_ERR_ARG.  v (np*3) may be NULL. */
int asg_load_particles_quantised(asg_ctx* ctx, const int* cell, const uint16_t* off,
                                 const float* v, int np, float left, float right, float cell_size,
                                 int grid);
int asg_load_particles_quantised_device(asg_ctx* ctx, const int* d_cell, const uint16_t* d_off,
                                        const float* d_v, int np, float left, float right,
                                        float cell_size, int grid);
/* One-shot form of asg_smooth for mixed-precision input (no halo marking):
 * rk and dens (host, np each, input order, may be NULL) receive the smoothing
 * length and the particle density; meshes and totals as in asg_smooth. */
int asg_smooth_quantised(asg_ctx* ctx, const int* cell, const uint16_t* off, const float* v,
                         int np, float left, float right, float cell_size, int grid, float boxsize,
                         const int* ncs, int n_nc, int sign, float* rk, float* dens,
                         float* const* meshes, double* totals);

/* ---- batched form ---------------------------------------------------------------
 * No counterpart in the reference, which runs one node-cube per MPI rank and
 * redshift: many cubes (or one cube at several redshifts) of uneven particle
 * counts run through the whole path in one CUDA graph.  Item i has np[i]
 * particles (with its shell) in [left[i], right[i]), box side boxsize[i];
 * every item gets the meshes ncs[0..n_nc-1] with the given sign.  The batch
 * owns device input and output arrays for all items.  The first
 * asg_batch_run plans (one eager pass that sizes every buffer and records
 * each item's pair count) and captures the per-item kernels into one graph;
 * later runs replay it.  Inputs whose pair counts outgrow the plan by more
 * than 1/16 are re-planned automatically.  Results equal asg_smooth's on each
 * item.  A batch uses its context exclusively until it is destroyed. */
typedef struct asg_batch asg_batch;
int asg_batch_create(asg_ctx* ctx, int n_items, const int* np, const int* np_local,
                     const float* left, const float* right, const float* boxsize, const int* ncs,
                     int n_nc, int sign, asg_batch** batch);
void asg_batch_destroy(asg_batch* batch);
/* Item positions x (np*3) and velocities v (np*3, may be NULL = 0), host or
 * device pointers. */
int asg_batch_set_item(asg_batch* batch, int item, const float* x, const float* v, int device_ptrs);
/* The mixed-precision form of an item (the batched asg_smooth_quantised):
 * cell (np int32 cell indices) and off (np*3 uint16 offsets) as for
 * asg_load_particles_quantised, in cells of side cell_size on a grid^3 grid
 * from the item's left; v as above.  The item keeps this form until
 * asg_batch_set_item gives it FP32 positions again. */
int asg_batch_set_item_quantised(asg_batch* batch, int item, const int* cell, const uint16_t* off,
                                 const float* v, float cell_size, int grid, int device_ptrs);
/* Run the items on `streams` concurrent streams (1..8, default 1): item i on
 * stream i % streams, each stream with its own scratch (about 300 bytes per
 * particle of the largest item), forked and joined inside the one graph. */
int asg_batch_set_streams(asg_batch* batch, int streams);
/* Optional autotuner: times the largest item with tree bucket sizes 16, 24, 32,
 * deposit work items of 2048, 4096, 8192 pairs, 2 or 4 warps per block of the
 * neighbour search and each deposit engine, and keeps the fastest; *leaf and
 * *seg receive the first two choices. */
int asg_batch_tune(asg_batch* batch, int* leaf, int* seg);
/* The batch's configuration (tuned or default): tree bucket size, deposit
 * work-item length, neighbour-search warps per block and the deposit engine
 * (1 or 2: tensor cores with one or two warps per tile item; 0: CUDA cores).
 * Any pointer may be NULL. */
int asg_batch_config(asg_batch* batch, int* leaf, int* seg, int* knn_warps, int* deposit_engine);
int asg_batch_run(asg_batch* batch);
/* Device time of the last graph launch (ms), kernels per launch, and the
 * interior particles of all items (the numerator of the batched metric). */
int asg_batch_stats(asg_batch* batch, double* graph_ms, long long* kernels,
                    long long* particles_local);
/* Results of one item: rk, dens (np each, input order), meshes[k] (6*nc^3),
 * totals (2 per mesh); any may be NULL. */
int asg_batch_get(asg_batch* batch, int item, float* rk, float* dens, float* const* meshes,
                  double* totals);

/* CUDA stream used by the context (cudaStream_t as void*). */
void* asg_stream(asg_ctx* ctx);
/* Count of kernels this library has launched so far (process-wide). */
long long asg_kernel_launches(asg_ctx* ctx);

/* ---- measurement ---------------------------------------------------------------- */
/* Phase timing with CUDA events on the context stream.  enable != 0 turns it on
 * and zeroes the accumulators; asg_phase_ms fills ms[0..ASG_NPHASES-1] with the
 * device time accumulated per phase since then. */
#define ASG_NPHASES 10
/* UPLOAD: the host-to-device copy of an end-to-end call's inputs; OUTPUT: from
 * the end of its last deposit until its copies to the host are done. */
enum { ASG_PH_INDEX = 0, ASG_PH_KNN = 1, ASG_PH_TIES = 2, ASG_PH_CHECK = 3, ASG_PH_DENS = 4,
       ASG_PH_DEPOSIT = 5, ASG_PH_HALOS = 6, ASG_PH_FOF = 7, ASG_PH_UPLOAD = 8,
       ASG_PH_OUTPUT = 9 };
int asg_set_timing(asg_ctx* ctx, int enable);
int asg_phase_ms(asg_ctx* ctx, double* ms);
const char* asg_phase_name(int phase);
/* Measured FP32 FMA throughput of this GPU (TFLOP/s, 2 flops per FMA) from a
 * register-resident FMA-chain kernel over all SMs: the FP32 roofline ceiling. */
int asg_measure_fp32_peak(asg_ctx* ctx, double* tflops);
/* Work statistics of the last deposit: (particle, 8^3-cell tile) pairs
 * deposited, mesh tiles, work items run. */
int asg_deposit_stats(asg_ctx* ctx, long long* pairs, long long* tiles, long long* items);

/* ---- allocation-free neighbour search -------------------------------------------- */
/* No counterpart in the reference: an entry point for callers that cannot
 * allocate device memory, for example a host application whose memory manager
 * reserves the whole GPU up front and lends libraries only its own buffers.
 * Same results as asg_neighbor_search (rk = sqrtf of the 33rd neighbour d2,
 * tent weights added to dens), but inputs and outputs are the caller's device
 * arrays: d_x (np*3 floats), d_rk (np floats, written), d_dens (np floats,
 * added to).  The scratch is a fixed array inside the library (about 10 MB),
 * so the call makes no cudaMalloc/cudaFree.  Limits: 33 <= np <=
 * ASG_NOALLOC_MAX_PARTICLES (larger inputs return ASG_ERR_NOALLOC_LIMIT).
 * All calls on one device share that scratch: calls that overlap on the GPU
 * race, so serialise them.
 * Preparing call: np = 0 with d_x, d_rk and d_dens all NULL loads the library's
 * module on the current device, which is when the scratch takes its device
 * memory (with CUDA's default lazy loading that is the first call on the
 * device, not the loading of the library), looks up the scratch's device
 * address and returns ASG_OK.  Make it on each device before reserving the
 * memory pool, and again after a cudaDeviceReset (the address kept from before
 * is stale then).  Without it the first search on a device does the same
 * set-up.
 * stream may be NULL (the default stream).  The call is synchronous: it waits
 * for its work on stream and reads the error word back before it returns, so
 * it cannot be captured into a CUDA graph.  It returns ASG_ERR_CUDA, before
 * doing any work, when the calling thread holds an unread CUDA error from
 * earlier work (left for the caller to read). */
#define ASG_NOALLOC_MAX_PARTICLES 32768
int asg_neighbor_search_noalloc(const float* d_x, int np, float left, float right, float* d_rk,
                                float* d_dens, void* stream);

#ifdef __cplusplus
}
#endif
#endif
