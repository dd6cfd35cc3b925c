// Block-sparse grid (8x8x8 blocks) device helpers.
//
// Per data block b: origin (3 int32), active mask (16 uint32, bit
// i + 8j + 64k), connectivity (27 uint32, entry (fx+1) + 3(fy+1) + 9(fz+1)).
// Field layout per block SoA: ((b * C + c) * 512 + i + 8j + 64k).
#pragma once
#include "common.cuh"

namespace ngb {

constexpr int kBlockVoxels = 512;

__device__ __forceinline__ bool bgrid_active(const uint32_t* __restrict__ mask, uint32_t b, int v)
{
    return (__ldg(mask + size_t(b) * 16 + (v >> 5)) >> (v & 31)) & 1u;
}

// Data block and in-block voxel of (i,j,k) + (ox,oy,oz) from block b, following
// bPartition::helpGetNghIdx (bPartition_imp.h:135-309); NGB_BGRID_NO_BLOCK if absent.
__device__ __forceinline__ uint32_t bgrid_ngh(const uint32_t* __restrict__ conn, uint32_t b, int i, int j, int k, int ox, int oy,
                                              int oz, int& v)
{
    int       ni = i + ox, nj = j + oy, nk = k + oz;
    const int fx = ni < 0 ? -1 : (ni >= 8 ? 1 : 0);
    const int fy = nj < 0 ? -1 : (nj >= 8 ? 1 : 0);
    const int fz = nk < 0 ? -1 : (nk >= 8 ? 1 : 0);
    uint32_t  nb = b;
    if (fx | fy | fz) {
        ni -= 8 * fx, nj -= 8 * fy, nk -= 8 * fz;
        nb = __ldg(conn + size_t(b) * 27 + (fx + 1) + 3 * (fy + 1) + 9 * (fz + 1));
    }
    v = ni + 8 * nj + 64 * nk;
    return nb;
}

// As bgrid_ngh, with this block's 27 connectivity entries already in `sconn`
// (shared memory): no dependent global load on the neighbour path.
__device__ __forceinline__ uint32_t bgrid_ngh_local(const uint32_t* sconn, uint32_t b, int i, int j, int k, int ox, int oy, int oz,
                                                    int& v)
{
    int       ni = i + ox, nj = j + oy, nk = k + oz;
    const int fx = ni < 0 ? -1 : (ni >= 8 ? 1 : 0);
    const int fy = nj < 0 ? -1 : (nj >= 8 ? 1 : 0);
    const int fz = nk < 0 ? -1 : (nk >= 8 ? 1 : 0);
    uint32_t  nb = b;
    if (fx | fy | fz) {
        ni -= 8 * fx, nj -= 8 * fy, nk -= 8 * fz;
        nb = sconn[(fx + 1) + 3 * (fy + 1) + 9 * (fz + 1)];
    }
    v = ni + 8 * nj + 64 * nk;
    return nb;
}

// Valid neighbour = block exists and voxel active (bPartition_imp.h:109-124).
__device__ __forceinline__ bool bgrid_valid_ngh(const uint32_t* __restrict__ mask, const uint32_t* __restrict__ conn, uint32_t b,
                                                int i, int j, int k, int ox, int oy, int oz, uint32_t& nb, int& v)
{
    nb = bgrid_ngh(conn, b, i, j, k, ox, oy, oz, v);
    return nb != NGB_BGRID_NO_BLOCK && bgrid_active(mask, nb, v);
}

int launch_bgrid_lbm(const ngb_bgrid_desc* d, const void* fin, void* fout, const uint32_t* flags, cudaStream_t s);

}  // namespace ngb
