/*
 * asmooth_oracle.h -- CPU oracle for the adaptive-smoothing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke test and the CPU-baseline leg of bench.py call it.  The product
 * path (libasmooth_gb300.so) never links or calls it.
 *
 * It is a plain-C restatement of the reference algorithm (junkoda/asmooth):
 *   - the "faithful" functions follow the reference step by step, including
 *     the midpoint kd-tree (KDTreeSimple), its traversal order, the float
 *     expression order of every distance / weight, and the serial
 *     accumulation order, so that their outputs are bit-identical to the
 *     reference built serially with -ffp-contract=off;
 *   - the "exact" functions compute the order-independent definitions the GPU
 *     path implements (exact top-33 by (d^2, index), exact FOF predicate);
 *   - the "64" outputs are FP64 restatements used for field error budgets.
 *
 * Positions are float[3] per particle, in input order.  All functions return
 * 0 on success and a negative code on a bad argument.
 */
#ifndef ASMOOTH_ORACLE_H
#define ASMOOTH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_K 33 /* KNeighbors::k (k_neighbors.h:47): 32 neighbours + self */

/* Faithful neighbour search: KDTreeSimple::construct (kdtree_balanced.cpp:212-296)
 * followed by neighbor_search for every particle in tree order
 * (clumping_tree_main.cpp:418-430, nbr_search.cpp:61-127).
 * rk[i]   <- sqrtf(d2 of the 33rd neighbour)            (input order)
 * dens[i] += tent weights scattered by the queries       (input order; accumulates)
 * nbr/nbr_d2 (optional, n*33): KNeighbors slots s[0..32] / x[0..32] per query as
 *   original indices (slot 0 = the 33rd, slot 32 = the nearest = self).
 * nthreads > 1 runs the query loop with OpenMP and atomic dens updates
 * (timing only: the summation order is then not the reference's). */
int orc_neighbor_search(const float* x, int n, float left, float right, int nthreads,
                        float* rk, float* dens, int* nbr, float* nbr_d2);

/* Exact k-nearest neighbours by the key (d2, original index), d2 computed with
 * the reference's float expression (nbr_search.cpp:20-25).
 * t33[i] = d2 of the 33rd key, idx33[i] = its index,
 * nbr (optional, n*33) = the 33 members sorted ascending by key. */
int orc_knn_exact(const float* x, int n, float left, float right, int nthreads,
                  float* t33, int* idx33, int* nbr);

/* dens from explicit 33-member lists (sorted ascending by key, as orc_knn_exact):
 * for every query p (input order) and its 32 nearest q (all but the 33rd),
 * dens32[q] += ker(p,q) in float (query order), dens64[q] += ker in FP64
 * (positions promoted to double, hinv = 1/(double)rk). rk_out = sqrtf(t33). */
int orc_dens_from_lists(const float* x, int n, const int* nbr, const float* t33,
                        float* rk_out, float* dens32, double* dens64);

/* Faithful mesh deposit: assign_on_mesh (coarse_mesh.cpp:45-127) when periodic=0,
 * assign_on_global_mesh (global_mesh.cpp:25-123) when periodic=1 (offset = rank
 * cube offset, 3 floats).  mesh (6*nc^3 floats, reference layout
 * [n | halo | c | v xyz interleaved]) is ADDED to (clear it first).
 * mesh64 (optional, 6*nc^3 doubles): the same cells with FP64 weights.
 * totals (optional, 2 doubles): FP64 sums of the library's cell weights (the
 * products of its float 1-D cell integrals, lib_weight) deposited into n and
 * into halo.
 * With mesh64 or totals the work runs over mesh planes in parallel (the float
 * mesh stays the serial loop's bit for bit); otherwise nthreads > 1 runs the
 * reference's OpenMP loop with atomics (timing only). */
int orc_assign_on_mesh(const float* x, const float* v, const float* dens, const float* rk,
                       const int* igrp, int n, float boxsize, int nc, int sign,
                       int periodic, const float* offset, int nthreads,
                       float* mesh, double* mesh64, double* totals);

/* n-channel-only variant (coarse_mesh.cpp:212-269). mesh has nc^3 floats. */
/* as orc_assign_on_mesh; mesh64, totals = FP64 sums of the library's cell weights */
int orc_assign_on_mesh_fw(const float* x, const float* v, const float* dens, const float* rk,
                          const int* igrp, int n, float boxsize, int nc, int sign, int periodic,
                          const float* offset, int nthreads, float* mesh, double* mesh64,
                          double* totals);
int orc_assign_on_density_mesh(const float* x, const float* rk, const int* igrp, int n,
                               float boxsize, int nc, int sign, float* mesh);

/* mesh_total (coarse_mesh.cpp:35-43): FP64 sum of the first nc^3 floats. */
double orc_mesh_total(const float* mesh, int nc);

/* write_mesh_separate normalisation (coarse_mesh.cpp:158-171), in place. */
int orc_normalise_mesh(float* mesh, int nc, float boxsize);

/* Faithful FOF: tree build + group_fof (fof.cpp:34-102).  igrp (input order) must
 * be 0 on entry; on return it holds the reference labels 1..ngroup.
 * exact=1 uses conservative AABB pruning instead of the reference's per-axis
 * float test, so every pair with d2 <= ll*ll is linked. */
int orc_group_fof(const float* x, int n, float left, float right, float ll, int exact,
                  int* igrp, int* ngroup);

/* remove_small_groups (fof.cpp:104-166): groups with >= 20 members -> 1..nhalo
 * in label order, all others -> 0. */
int orc_remove_small_groups(int* igrp, int n, int ngrp, int* nhalo);

/* Zipped particle decode of read_pm_file_zip (file_reader2.cpp:187-252). */
int orc_decode_zip(const unsigned char* off, const short* vel, const unsigned char* counts8,
                   const int* counts32, int n32, int np_local, int nc, int mesh_scale, float v_r2i,
                   const float* shift, float* x, float* v);

/* FOF halo catalogue of write_fof_halos (fof.cpp:169-219): out gets up to
 * nhalo records {x[3], v[3], int nfof} (7 words), *nlocal of them kept. */
int orc_fof_halos(const float* x, const float* v, const int* igrp, int n, int nhalo,
                  float boxsize, float* out, int* nlocal);

/* Faithful SO-halo marking: the loop at clumping_tree_main.cpp:474-485 around
 * mark_halo_particles (nbr_search.cpp:140-165).  halos: 5 floats per halo
 * (x, y, z, r, mass) = struct Halo (basic_types.h:17-20).  Halos whose centre is
 * strictly inside (left,right)^3 mark every particle with d2 < r*r (igrp=-1).
 * np_halo = sum of per-halo counts, m_halo = sum of mass/8. exact=1: AABB pruning. */
int orc_mark_halo_particles(const float* x, int n, float left, float right,
                            const float* halos, int nh, int exact,
                            int* igrp, long* np_halo, double* m_halo);

#ifdef __cplusplus
}
#endif
#endif
