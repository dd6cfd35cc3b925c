// ORACLE — test infrastructure only.
//
// CPU restatement of Neon's block-sparse bGrid construction for a single
// partition, and of its neighbour lookup. Used by the tests as the checker;
// the product library never links it.
//
// Follows (paths relative to the Neon repository):
//   libNeonDomain/include/Neon/domain/tools/partitioning/SpanDecomposition.h:71-96
//       a block is counted iff one voxel of it is inside the domain and active
//   libNeonDomain/include/Neon/domain/tools/partitioning/SpanClassifier.h:170-191, 228-237
//       single partition: blocks are appended scanning bz, then by, then bx (x fastest)
//   libNeonDomain/src/domain/tools/partitioning/SpanClassifier.cpp:7-20
//       the data-block index is the rank of the block in that scan
//   libNeonDomain/include/Neon/domain/tools/Partitioner1D.h:212-255
//       block origin = block 3-D index * 8
//   libNeonDomain/include/Neon/domain/details/bGrid/bGrid_imp.h:80-136
//       per-block 512-bit active mask, bit x + 8y + 64z (StaticBlock.h:79-98)
//   libNeonDomain/include/Neon/domain/details/bGrid/bGrid_imp.h:139-172
//       27-entry block connectivity, entry i + 3j + 9k -> block at (i-1, j-1, k-1),
//       UINT32_MAX when absent; the centre entry is the block itself
//   libNeonDomain/include/Neon/domain/details/bGrid/bPartition_imp.h:95-124, 135-309
//       per-block SoA addressing and neighbour resolution
#pragma once
#include <cstdint>
#include <vector>
#include <algorithm>

namespace oracle {

struct BGrid {
    int                   nx = 0, ny = 0, nz = 0;     // domain
    int                   bnx = 0, bny = 0, bnz = 0;  // blocks per axis (ceil(dim / 8))
    uint32_t              nBlocks = 0;
    uint64_t              nActiveVoxels = 0;
    std::vector<int32_t>  origin;   // 3 per block
    std::vector<uint32_t> mask;     // 16 words per block
    std::vector<uint32_t> conn;     // 27 per block
    std::vector<int64_t>  blockOf;  // dense block grid -> data-block index or -1
};

static constexpr uint32_t kNoBlock = 0xffffffffu;

// active: dense nx*ny*nz bytes, x fastest; non-zero = active voxel.
inline BGrid bgrid_build(int nx, int ny, int nz, const uint8_t* active)
{
    BGrid g;
    g.nx = nx, g.ny = ny, g.nz = nz;
    g.bnx = (nx + 7) / 8, g.bny = (ny + 7) / 8, g.bnz = (nz + 7) / 8;
    g.blockOf.assign(size_t(g.bnx) * g.bny * g.bnz, -1);
    for (int bz = 0; bz < g.bnz; bz++)
        for (int by = 0; by < g.bny; by++)
            for (int bx = 0; bx < g.bnx; bx++) {
                uint32_t words[16] = {0};
                uint32_t count = 0;
                for (int k = 0; k < 8; k++)
                    for (int j = 0; j < 8; j++)
                        for (int i = 0; i < 8; i++) {
                            const int x = bx * 8 + i, y = by * 8 + j, z = bz * 8 + k;
                            if (x >= nx || y >= ny || z >= nz) continue;
                            if (!active[size_t(x) + size_t(nx) * (size_t(y) + size_t(ny) * z)]) continue;
                            const uint32_t bit = uint32_t(i + 8 * j + 64 * k);
                            words[bit >> 5] |= 1u << (bit & 31u);
                            count++;
                        }
                if (count == 0) continue;
                g.blockOf[size_t(bx) + size_t(g.bnx) * (size_t(by) + size_t(g.bny) * bz)] = g.nBlocks;
                g.origin.push_back(bx * 8);
                g.origin.push_back(by * 8);
                g.origin.push_back(bz * 8);
                for (int w = 0; w < 16; w++) g.mask.push_back(words[w]);
                g.nActiveVoxels += count;
                g.nBlocks++;
            }
    g.conn.assign(size_t(g.nBlocks) * 27, kNoBlock);
    for (uint32_t b = 0; b < g.nBlocks; b++) {
        const int bx = g.origin[3 * b] / 8, by = g.origin[3 * b + 1] / 8, bz = g.origin[3 * b + 2] / 8;
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) {
                    const int nbx = bx + i - 1, nby = by + j - 1, nbz = bz + k - 1;
                    uint32_t  v = kNoBlock;
                    if (nbx >= 0 && nby >= 0 && nbz >= 0 && nbx < g.bnx && nby < g.bny && nbz < g.bnz) {
                        const int64_t id = g.blockOf[size_t(nbx) + size_t(g.bnx) * (size_t(nby) + size_t(g.bny) * nbz)];
                        if (id >= 0) v = uint32_t(id);
                    }
                    g.conn[size_t(b) * 27 + i + 3 * j + 9 * k] = v;
                }
    }
    return g;
}

inline bool bgrid_is_active(const BGrid& g, uint32_t block, int i, int j, int k)
{
    const uint32_t bit = uint32_t(i + 8 * j + 64 * k);
    return (g.mask[size_t(block) * 16 + (bit >> 5)] >> (bit & 31u)) & 1u;
}

// Neighbour resolution of bPartition::helpGetNghIdx + helpNghPitch: returns the
// (block, in-block voxel) of (i,j,k)+off, or false when the neighbour block is
// absent or the voxel is not active.
inline bool bgrid_ngh(const BGrid& g, uint32_t block, int i, int j, int k, int ox, int oy, int oz,
                      uint32_t& nb, int& ni, int& nj, int& nk)
{
    ni = i + ox, nj = j + oy, nk = k + oz;
    const int fx = ni < 0 ? -1 : (ni >= 8 ? 1 : 0);
    const int fy = nj < 0 ? -1 : (nj >= 8 ? 1 : 0);
    const int fz = nk < 0 ? -1 : (nk >= 8 ? 1 : 0);
    nb = block;
    if (fx | fy | fz) {
        ni -= fx * 8, nj -= fy * 8, nk -= fz * 8;
        nb = g.conn[size_t(block) * 27 + (fx + 1) + 3 * (fy + 1) + 9 * (fz + 1)];
        if (nb == kNoBlock) return false;
    }
    return bgrid_is_active(g, nb, ni, nj, nk);
}

// Per-block SoA pitch (bPartition_imp.h:95-107).
inline size_t bgrid_pitch(uint32_t block, int card, int C, int i, int j, int k)
{
    return (size_t(block) * C + card) * 512 + size_t(i + 8 * j + 64 * k);
}

}  // namespace oracle
