/*
 * ref_harness.cpp -- thin C entry points around the REFERENCE's own hot-path
 * functions (junkoda/asmooth), compiled in place from the reference sources by
 * oracle/build_ref.sh into oracle/_ref/.  TEST INFRASTRUCTURE ONLY: used to pin
 * the C restatement (asmooth_oracle.c) and to generate golden fixtures.
 *
 * Each entry point replays one reference call site on arrays supplied by the
 * caller and un-permutes the kd-tree's in-place reordering so that outputs are
 * in input order.  The reference is built serially (no OpenMP) with
 * -ffp-contract=off for parity; a second build with -fopenmp is timed only.
 */
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "basic_types.h"
#include "coarse_mesh.h"
#include "exchange_buffer.h"
#include "file_reader2.h"
#include "fof.h"
#include "k_neighbors.h"
#include "kdtree_balanced.h"
#include "mpi_interface.h"
#include "nbr_search.h"

int asg_shim_coords[3] = {0, 0, 0};

/* defined in global_mesh.cpp; the reference declares it in no header */
void assign_on_global_mesh(Particles const* const particles, MpiInterface const* const mpi,
                           float mesh[], const int nc, const int sign);

static Particles* make_particles(int n)
{
    Particles* ps = new Particles();
    ps->allocate(n + 1);
    ps->np_local = n;
    ps->np_with_buffers = n;
    ps->np_total = n;
    for (int i = 0; i < n; ++i) {
        Particle& p = ps->particle[i];
        p.x[0] = p.x[1] = p.x[2] = 0.0f;
        p.v[0] = p.v[1] = p.v[2] = 0.0f;
        p.dens = p.rk = 0.0f;
        p.igrp = 0;
    }
    return ps;
}

static void free_particles(Particles* ps)
{
    std::free(ps->particle);
    ps->particle = 0;
    delete ps;
}

static KDTree* make_tree(Particles* ps, float left, float right)
{
    KDTree* tree = new KDTreeSimple();
    /* node storage is unchecked in the reference (kdtree_balanced.cpp:208):
     * size it far above what a midpoint tree of n particles can need */
    tree->allocate(std::max(64 * ps->np_with_buffers, 4096), 16);
    tree->construct(ps, left, right);
    return tree;
}

extern "C" {

/* clumping_tree_main.cpp:390-395 + :418-430 (serial) */
int ref_neighbor_search(const float* x, int n, float left, float right,
                        float* rk, float* dens, int* nbr, float* nbr_d2)
{
    Particles* ps = make_particles(n);
    Particle* p = ps->particle;
    for (int i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) p[i].x[d] = x[3 * i + d];
        p[i].dens = dens[i];
        p[i].igrp = i; /* carries the input index through the permutation */
    }
    KDTree* tree = make_tree(ps, left, right);
    set_nbr_search(tree->root(), ps->particle);
    KNeighbors knbrs;
    for (int i = 0; i < n; ++i) {
        neighbor_search(p + i, &knbrs);
        if (nbr) {
            for (int s = 0; s < KNeighbors::k; ++s) {
                nbr[(size_t)p[i].igrp * KNeighbors::k + s] = knbrs.nbr(s)->igrp;
                if (nbr_d2) nbr_d2[(size_t)p[i].igrp * KNeighbors::k + s] = knbrs.r2(s);
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        rk[p[i].igrp] = p[i].rk;
        dens[p[i].igrp] = p[i].dens;
    }
    delete tree;
    free_particles(ps);
    return 0;
}

static Particles* particles_from(const float* x, const float* v, const float* dens,
                                 const float* rk, const int* igrp, int n, float boxsize)
{
    Particles* ps = make_particles(n);
    ps->boxsize = boxsize;
    for (int i = 0; i < n; ++i) {
        Particle& q = ps->particle[i];
        for (int d = 0; d < 3; ++d) {
            q.x[d] = x[3 * i + d];
            q.v[d] = v ? v[3 * i + d] : 0.0f;
        }
        q.dens = dens ? dens[i] : 0.0f;
        q.rk = rk ? rk[i] : 0.0f;
        q.igrp = igrp ? igrp[i] : 0;
    }
    return ps;
}

/* clear_mesh + assign_on_mesh (coarse_mesh.cpp:24-127), particles in input order */
int ref_assign_on_mesh(const float* x, const float* v, const float* dens, const float* rk,
                       const int* igrp, int n, float boxsize, int nc, int sign, float* mesh)
{
    Particles* ps = particles_from(x, v, dens, rk, igrp, n, boxsize);
    clear_mesh(mesh, nc);
    assign_on_mesh(ps, mesh, nc, sign);
    free_particles(ps);
    return 0;
}

/* assign_on_global_mesh (global_mesh.cpp:25-123) for a rank at grid coords[] */
int ref_assign_on_global_mesh(const float* x, const float* v, const float* dens, const float* rk,
                              const int* igrp, int n, float boxsize, int nc, int sign,
                              const int* coords, float* mesh)
{
    for (int d = 0; d < 3; ++d) asg_shim_coords[d] = coords ? coords[d] : 0;
    MpiInterface* mpi = new MpiInterface();
    Particles* ps = particles_from(x, v, dens, rk, igrp, n, boxsize);
    clear_mesh(mesh, nc);
    assign_on_global_mesh(ps, mpi, mesh, nc, sign);
    free_particles(ps);
    delete mpi;
    for (int d = 0; d < 3; ++d) asg_shim_coords[d] = 0;
    return 0;
}

/* assign_on_density_mesh (coarse_mesh.cpp:212-269); mesh has nc^3 floats */
int ref_assign_on_density_mesh(const float* x, const float* rk, const int* igrp, int n,
                               float boxsize, int nc, int sign, float* mesh)
{
    Particles* ps = particles_from(x, 0, 0, rk, igrp, n, boxsize);
    for (size_t j = 0; j < (size_t)nc * nc * nc; ++j) mesh[j] = 0.0f;
    assign_on_density_mesh(ps, mesh, nc, sign);
    free_particles(ps);
    return 0;
}

double ref_mesh_total(const float* mesh, int nc) { return mesh_total(mesh, nc); }

/* write_mesh_separate (coarse_mesh.cpp:147-208): normalises mesh in place and
 * writes <base>{n,h,c,vel}<inode>.dat */
int ref_write_mesh_separate(const char* base, int inode, float* mesh, int nc, float boxsize)
{
    write_mesh_separate(base, inode, mesh, nc, boxsize);
    return 0;
}

/* The single-rank periodic shell: exchange_buffer (exchange_buffer.cpp:13-168)
 * on one rank of a 1x1x1 periodic grid, every direction a self-exchange, then
 * the filter of remove_extra_particles (clumping_tree_main.cpp:550-576, a
 * static function of the driver, replayed here).  Out arrays hold cap
 * particles; returns -1 when they are too small. */
int ref_exchange_buffer(const float* x, const float* v, int n, float boxsize, float buffer_factor,
                        float* out_x, float* out_v, int cap, int* n_with, int* n_local)
{
    const int alloc = 8 * n + 1024;  /* the shell is at most 26/27 x 7 copies */
    Particles* ps = make_particles(alloc);
    ps->np_local = n;
    ps->np_with_buffers = n;
    ps->np_allocated = alloc;
    ps->boxsize = boxsize;
    Particle* p = ps->particle;
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            p[i].x[d] = x[3 * i + d];
            p[i].v[d] = v[3 * i + d];
        }
    MpiInterface mpi;
    exchange_buffer(&mpi, ps, buffer_factor);
    /* remove_extra_particles */
    const float dx = buffer_factor * ps->boxsize;
    const float left = -dx, right = ps->boxsize + dx;
    int kept = 0, local = n;
    for (int i = 0; i < ps->np_with_buffers; ++i) {
        const Particle& q = p[i];
        if (left < q.x[0] && q.x[0] < right && left < q.x[1] && q.x[1] < right && left < q.x[2] &&
            q.x[2] < right) {
            if (kept >= cap) { free_particles(ps); return -1; }
            for (int d = 0; d < 3; ++d) {
                out_x[3 * kept + d] = q.x[d];
                out_v[3 * kept + d] = q.v[d];
            }
            ++kept;
        } else if (i < n) {
            --local;
        }
    }
    *n_with = kept;
    *n_local = local;
    free_particles(ps);
    return 0;
}

/* read_pm_file_xv / read_pm_file_zip (file_reader2.cpp:24-86, :90-272): the
 * particles of <filebase><inode>/<redshift>{xv,zip0..3_}<inode>.dat, up to cap */
static int copy_out(Particles* ps, float* x, float* v, int cap, int* np)
{
    const int n = (int)ps->np_local;
    if (n > cap) return -1;
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            x[3 * i + d] = ps->particle[i].x[d];
            v[3 * i + d] = ps->particle[i].v[d];
        }
    *np = n;
    return 0;
}

int ref_read_pm_file_xv(const char* filebase, const char* redshift, int inode, const float* shift,
                        int cap, float* x, float* v, int* np)
{
    Particles* ps = make_particles(cap + 8);
    read_pm_file_xv(filebase, redshift, inode, 0.0f, shift, ps);
    const int r = copy_out(ps, x, v, cap, np);
    free_particles(ps);
    return r;
}

int ref_read_pm_file_zip(const char* filebase, const char* redshift, int inode, int nc_node_dim,
                         int mesh_scale, const float* shift, int cap, float* x, float* v, int* np,
                         float* boxsize)
{
    Particles* ps = make_particles(cap + 8);
    read_pm_file_zip(filebase, redshift, inode, 0.0f, nc_node_dim, mesh_scale, shift, ps);
    *boxsize = ps->boxsize;
    const int r = copy_out(ps, x, v, cap, np);
    free_particles(ps);
    return r;
}

/* write_mesh (coarse_mesh.cpp:128-143): int nc, int dof, float boxsize, mesh */
int ref_write_mesh(const char* filename, float* mesh, int nc, float boxsize)
{
    write_mesh(const_cast<char*>(filename), mesh, nc, boxsize);
    return 0;
}

/* write_fof_halos (fof.cpp:169-219) on particles in the caller's order, with a
 * zeroed work buffer (the function never clears v[2] itself) */
int ref_write_fof_halos(const char* filename, const float* x, const float* v, const int* igrp,
                        int n, int nhalo, float boxsize)
{
    Particles* ps = make_particles(n);
    ps->boxsize = boxsize;
    Particle* p = ps->particle;
    for (int i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) {
            p[i].x[d] = x[3 * i + d];
            p[i].v[d] = v[3 * i + d];
        }
        p[i].igrp = igrp[i];
    }
    const size_t words = std::max((size_t)n, 7 * ((size_t)nhalo + 2));
    float* buf = (float*)std::calloc(words, sizeof(float));
    write_fof_halos(filename, ps, buf, nhalo);
    std::free(buf);
    free_particles(ps);
    return 0;
}

/* clumping_tree_main.cpp:392-407: tree, group_fof, remove_small_groups */
int ref_group_fof(const float* x, int n, float left, float right, float ll,
                  int* igrp, int* ngroup)
{
    Particles* ps = make_particles(n);
    Particle* p = ps->particle;
    for (int i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) p[i].x[d] = x[3 * i + d];
        p[i].v[0] = (float)i; /* input index, exact below 2^24 */
        p[i].igrp = 0;
    }
    KDTree* tree = make_tree(ps, left, right);
    *ngroup = group_fof(ps, tree, ll);
    for (int i = 0; i < n; ++i) igrp[(int)p[i].v[0]] = p[i].igrp;
    delete tree;
    free_particles(ps);
    return 0;
}

int ref_remove_small_groups(int* igrp, int n, int ngrp, int* nhalo)
{
    Particles* ps = make_particles(n);
    for (int i = 0; i < n; ++i) ps->particle[i].igrp = igrp[i];
    int* buf = (int*)std::malloc(sizeof(int) * ((size_t)ngrp + 1));
    *nhalo = remove_small_groups(ps, buf, ngrp);
    for (int i = 0; i < n; ++i) igrp[i] = ps->particle[i].igrp;
    std::free(buf);
    free_particles(ps);
    return 0;
}

/* clumping_tree_main.cpp:465-485: mark every SO halo whose centre is inside */
int ref_mark_halo_particles(const float* x, int n, float left, float right,
                            const float* halos, int nh, int* igrp, long* np_halo, double* m_halo)
{
    Particles* ps = make_particles(n);
    Particle* p = ps->particle;
    for (int i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) p[i].x[d] = x[3 * i + d];
        p[i].v[0] = (float)i;
        p[i].igrp = igrp[i];
    }
    KDTree* tree = make_tree(ps, left, right);
    set_nbr_search(tree->root(), ps->particle);
    const Halo* h = reinterpret_cast<const Halo*>(halos);
    long np = 0;
    double mh = 0.0;
    for (int i = 0; i < nh; ++i) {
        if (left < h[i].x[0] && h[i].x[0] < right && left < h[i].x[1] && h[i].x[1] < right &&
            left < h[i].x[2] && h[i].x[2] < right) {
            np += mark_halo_particles(tree->root(), h[i].x, h[i].r);
            mh += h[i].mass / 8.0f;
        }
    }
    for (int i = 0; i < n; ++i) igrp[(int)p[i].v[0]] = p[i].igrp;
    *np_halo = np;
    *m_halo = mh;
    delete tree;
    free_particles(ps);
    return 0;
}

} /* extern "C" */
