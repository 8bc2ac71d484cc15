// asg_output.cu -- the outputs of the path: the FOF halo catalogue
// (write_fof_halos, fof.cpp:169-219) computed on the device, and the byte
// formats of the mesh and catalogue files (write_mesh, coarse_mesh.cpp:128-143;
// write_mesh_separate, coarse_mesh.cpp:147-208; write_fof_halos).
//
// Catalogue: per label 1..nhalo, the float sums of x and v over the members in
// the caller's array order (one thread per halo adds them sequentially, as the
// reference's loop does, so the sums are the reference's bits), divided by the
// member count; halos whose centre is strictly inside (0, boxsize)^3 are kept
// in label order.  The members are grouped by a radix sort of
// (label << 32 | input index).
#include <cstdio>
#include <string>

#include "../../include/asmooth_gb300.h"
#include "asg_common.cuh"
#include "asg_internal.h"

namespace asg {

constexpr int REC_WORDS = 7;  // struct FofHalo (fof.cpp:22-25): float x[3], v[3]; int nfof

static size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

struct CatLayout {
    size_t keys0, keys1, vals0, vals1, sort_tmp, start, end, rec, flags, scan_tmp, total;
};

static CatLayout cat_layout(int n, int nhalo)
{
    CatLayout L{};
    const size_t N = (size_t)n, H = (size_t)nhalo + 1;
    size_t o = 0;
    auto take = [&](size_t b) {
        const size_t at = o;
        o = al256(o + b);
        return at;
    };
    L.keys0 = take(8 * N);
    L.keys1 = take(8 * N);
    L.vals0 = take(4 * N);
    L.vals1 = take(4 * N);
    L.sort_tmp = take(radix_sort_temp_bytes(n));
    L.start = take(4 * H);
    L.end = take(4 * H);
    L.rec = take(4 * REC_WORDS * H);
    L.flags = take(4 * H);
    L.scan_tmp = take(scan_temp_bytes(H));
    L.total = o;
    return L;
}

size_t fof_catalogue_bytes(int n, int nhalo) { return cat_layout(n, nhalo).total; }

__global__ void k_cat_keys(const float4* __restrict__ pos, const int* __restrict__ igrp, int n,
                           int w_index, int nhalo, uint64_t* __restrict__ keys, int* __restrict__ vals)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int lab = igrp[j];
    const uint32_t idx = w_index ? (uint32_t)__float_as_int(pos[j].w) : (uint32_t)j;
    const uint64_t hi = (lab >= 1 && lab <= nhalo) ? (uint64_t)lab : 0u;
    keys[j] = (hi << 32) | idx;
    vals[j] = j;
}

__global__ void k_cat_bounds(const uint64_t* __restrict__ keys, int n, uint32_t* __restrict__ start,
                             uint32_t* __restrict__ end)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const uint32_t lab = (uint32_t)(keys[m] >> 32);
    if (lab == 0) return;
    if (m == 0 || (uint32_t)(keys[m - 1] >> 32) != lab) start[lab] = (uint32_t)m;
    if (m == n - 1 || (uint32_t)(keys[m + 1] >> 32) != lab) end[lab] = (uint32_t)m + 1;
}

// one thread per halo: sequential float sums in member (= caller array) order
__global__ void k_cat_sums(const float4* __restrict__ pos, const float4* __restrict__ vel,
                           const int* __restrict__ order, const uint32_t* __restrict__ start,
                           const uint32_t* __restrict__ end, int nhalo, float boxsize,
                           float* __restrict__ rec, uint32_t* __restrict__ flags)
{
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nhalo) return;
    const uint32_t s = start[h + 1], e = end[h + 1];
    float sx = 0.f, sy = 0.f, sz = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
#pragma unroll 4
    for (uint32_t m = s; m < e; ++m) {
        const int j = order[m];
        const float4 p = pos[j];
        const float4 v = vel[j];
        sx = __fadd_rn(sx, p.x);
        sy = __fadd_rn(sy, p.y);
        sz = __fadd_rn(sz, p.z);
        ux = __fadd_rn(ux, v.x);
        uy = __fadd_rn(uy, v.y);
        uz = __fadd_rn(uz, v.z);
    }
    const int nf = (int)(e - s);
    const float fn = __int2float_rn(nf);
    float r[6] = {__fdiv_rn(sx, fn), __fdiv_rn(sy, fn), __fdiv_rn(sz, fn),
                  __fdiv_rn(ux, fn), __fdiv_rn(uy, fn), __fdiv_rn(uz, fn)};
    float* o = rec + (size_t)REC_WORDS * h;
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = r[k];
    o[6] = __int_as_float(nf);
    flags[h] = (0.0f < r[0] && r[0] < boxsize && 0.0f < r[1] && r[1] < boxsize && 0.0f < r[2] &&
                r[2] < boxsize) ? 1u : 0u;
}

// scan: exclusive scan of the keep flags over nhalo + 1 entries (the last flag
// is 0), so halo h is kept when scan[h + 1] > scan[h] and scan[nhalo] is the count
__global__ void k_cat_compact(const float* __restrict__ rec, const uint32_t* __restrict__ scan,
                              int nhalo, float* __restrict__ out, uint32_t* __restrict__ nlocal)
{
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h == 0) *nlocal = scan[nhalo];
    if (h >= nhalo || scan[h + 1] == scan[h]) return;
    const float* a = rec + (size_t)REC_WORDS * h;
    float* b = out + (size_t)REC_WORDS * scan[h];
#pragma unroll
    for (int k = 0; k < REC_WORDS; ++k) b[k] = a[k];
}

void launch_fof_catalogue(const float4* pos, const float4* vel, const int* igrp, int n, int w_index,
                          int nhalo, float boxsize, void* scratch, float* out, uint32_t* nlocal,
                          cudaStream_t s)
{
    const CatLayout L = cat_layout(n, nhalo);
    unsigned char* b = static_cast<unsigned char*>(scratch);
    auto U64 = [&](size_t o) { return reinterpret_cast<uint64_t*>(b + o); };
    auto I = [&](size_t o) { return reinterpret_cast<int*>(b + o); };
    auto U = [&](size_t o) { return reinterpret_cast<uint32_t*>(b + o); };
    const size_t H = (size_t)nhalo + 1;
    cudaMemsetAsync(b + L.start, 0, 4 * H, s);
    cudaMemsetAsync(b + L.end, 0, 4 * H, s);
    cudaMemsetAsync(b + L.flags, 0, 4 * H, s);
    if (n > 0) {
        k_cat_keys<<<(n + 255) / 256, 256, 0, s>>>(pos, igrp, n, w_index, nhalo, U64(L.keys0),
                                                    I(L.vals0));
        int bits = 32;
        while (bits < 64 && ((uint64_t)nhalo >> (bits - 32)) != 0) ++bits;
        const int cur = radix_sort(U64(L.keys0), I(L.vals0), U64(L.keys1), I(L.vals1), n, bits,
                                   b + L.sort_tmp, s);
        const uint64_t* keys = U64(cur ? L.keys1 : L.keys0);
        const int* order = I(cur ? L.vals1 : L.vals0);
        k_cat_bounds<<<(n + 255) / 256, 256, 0, s>>>(keys, n, U(L.start), U(L.end));
        count_launches(2);
        if (nhalo > 0) {
            k_cat_sums<<<(nhalo + 127) / 128, 128, 0, s>>>(pos, vel, order, U(L.start), U(L.end),
                                                           nhalo, boxsize,
                                                           reinterpret_cast<float*>(b + L.rec),
                                                           U(L.flags));
            count_launches(1);
        }
    }
    exclusive_scan_u32(U(L.flags), H, b + L.scan_tmp, s);  // in place: flags -> offsets
    k_cat_compact<<<(unsigned)((H + 255) / 256), 256, 0, s>>>(
        reinterpret_cast<const float*>(b + L.rec), U(L.flags), nhalo, out, nlocal);
    count_launches(1);
}

// ---- file formats (host) ----------------------------------------------------------

// int nc, then the floats (one file of write_mesh_separate, coarse_mesh.cpp:180-206)
static int write_block(const std::string& name, int nc, const float* data, size_t count)
{
    FILE* fp = std::fopen(name.c_str(), "wb");
    if (!fp) return ASG_ERR_IO;
    bool ok = std::fwrite(&nc, sizeof(int), 1, fp) == 1;
    ok = ok && std::fwrite(data, sizeof(float), count, fp) == count;
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? ASG_OK : ASG_ERR_IO;
}

// <base>{n,h,c,vel}<inode>.dat of an already normalised mesh [n | halo | c | v xyz]
int write_mesh_files(const char* base, int inode, const float* mesh, int nc)
{
    const size_t nm = (size_t)nc * nc * nc;
    const std::string b(base), i = std::to_string(inode) + ".dat";
    if (int r = write_block(b + "n" + i, nc, mesh, nm)) return r;
    if (int r = write_block(b + "h" + i, nc, mesh + nm, nm)) return r;
    if (int r = write_block(b + "c" + i, nc, mesh + 2 * nm, nm)) return r;
    return write_block(b + "vel" + i, nc, mesh + 3 * nm, 3 * nm);
}

// int nlocal, int sizeof(FofHalo) = 28, the records, int nlocal (fof.cpp:210-217)
int write_fof_file(const char* filename, const float* rec, int nlocal)
{
    FILE* fp = std::fopen(filename, "wb");
    if (!fp) return ASG_ERR_IO;
    const int size_halo = 4 * REC_WORDS;
    bool ok = std::fwrite(&nlocal, sizeof(int), 1, fp) == 1;
    ok = ok && std::fwrite(&size_halo, sizeof(int), 1, fp) == 1;
    ok = ok && std::fwrite(rec, 4 * REC_WORDS, (size_t)nlocal, fp) == (size_t)nlocal;
    ok = ok && std::fwrite(&nlocal, sizeof(int), 1, fp) == 1;
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? ASG_OK : ASG_ERR_IO;
}

}  // namespace asg

// write_mesh (coarse_mesh.cpp:128-143): int nc, int dof = 6, float boxsize, 6*nc^3 floats
extern "C" int asg_write_mesh(const char* filename, const float* mesh, int nc, float boxsize)
{
    if (!filename || !mesh || nc <= 0 || nc > 1290) return ASG_ERR_ARG;
    FILE* fp = std::fopen(filename, "wb");
    if (!fp) return ASG_ERR_IO;
    const int dof = 6;
    const size_t count = (size_t)dof * nc * nc * nc;
    bool ok = std::fwrite(&nc, sizeof(int), 1, fp) == 1;
    ok = ok && std::fwrite(&dof, sizeof(int), 1, fp) == 1;
    ok = ok && std::fwrite(&boxsize, sizeof(float), 1, fp) == 1;
    ok = ok && std::fwrite(mesh, sizeof(float), count, fp) == count;
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? ASG_OK : ASG_ERR_IO;
}

namespace asg {

}  // namespace asg
