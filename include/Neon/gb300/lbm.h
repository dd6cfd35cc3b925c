// Named LBM containers backed by the sm_103a kernels of the C ABI.
//
// Drop-in replacements for the containers of
// benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h: an application keeps
// its grids, fields and Skeleton and swaps LbmContainers<...>::iteration /
// computeWallNghMask for these. Population fields hold `double` or `float`
// (f), or `__nv_bfloat16` (g = f - w) / `__half` (2^14 (f - w), NGB_F16OFF_SCALE); the cell-type field holds
// one uint32 per cell in the packed form NGB_MAKE_FLAG(mask, classification)
// (CellType.h:3-35 values for the classification).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <array>
#include <type_traits>

#include "Neon/domain/bGrid.h"
#include "Neon/domain/dGrid.h"
#include "neon_gb300.h"

namespace Neon {
namespace gb300 {

template <typename T>
constexpr int storage_of()
{
    if constexpr (std::is_same_v<T, double>) return NGB_STORE_F64;
    if constexpr (std::is_same_v<T, float>) return NGB_STORE_F32;
    if constexpr (std::is_same_v<T, __half>) return NGB_STORE_F16OFF;
    if constexpr (std::is_same_v<T, __nv_bfloat16>) return NGB_STORE_BF16OFF;
    return -1;
}

// Wall terms: the population a wall node holds, by its class ([0] bounce-back, [1] moving wall).
struct WallTerms {
    std::array<double, 27> bounceBack{};
    std::array<double, 27> movingWall{};
};

// The stream-collide container of LbmTools.h:284-325 on dGrid or bGrid.
// Q = 19 (D3Q19) or 27 (D3Q27); fIn/fOut have cardinality Q.
template <int Q, typename PopField, typename FlagField>
auto iteration(const PopField& fIn, const FlagField& flags, double omega, const WallTerms& walls, PopField& fOut)
    -> set::Container
{
    using T = typename PopField::Type;
    static_assert(storage_of<T>() >= 0, "population type must be double, float, __half or __nv_bfloat16");
    static_assert(std::is_same_v<typename FlagField::Type, uint32_t>, "cell-type field must hold packed uint32 flags");
    static_assert(Q == 19 || Q == 27, "Q must be 19 or 27");
    const T*        in = fIn.mem();
    T*              out = fOut.mem();
    const uint32_t* fl = flags.mem();
    if constexpr (std::is_same_v<typename PopField::Grid, Neon::dGrid>) {
        const int32_3d     d = fIn.getDimension();
        ngb_lbm_dense_desc desc{};
        desc.nx = d.x, desc.ny = d.y, desc.nz = d.z, desc.q = Q, desc.storage = storage_of<T>(), desc.box_cavity = 0;
        desc.plane_stride = 0, desc.omega = omega;
        for (int k = 0; k < 27; k++) desc.wall_term[0][k] = walls.bounceBack[k], desc.wall_term[1][k] = walls.movingWall[k];
        return set::Container("LBM_iteration", fIn.getBackend(), [desc, in, out, fl]() -> set::Launch {
            set::Launch l;
            l.signature = set::bytes_of(desc);
            l.run = [desc, in, out, fl](cudaStream_t s) { NEON_NGB_CHECK(ngb_lbm_dense_step(&desc, in, out, fl, s)); };
            return l;
        });
    } else {
        const auto&    B = fIn.getGrid().getBlocks();
        ngb_bgrid_desc desc{};
        desc.n_blocks = int32_t(B.nBlocks), desc.q = Q, desc.storage = storage_of<T>(), desc.omega = omega;
        for (int k = 0; k < 27; k++) desc.wall_term[0][k] = walls.bounceBack[k], desc.wall_term[1][k] = walls.movingWall[k];
        desc.origin = B.dOrigin, desc.mask = B.dMask, desc.conn = B.dConn;
        return set::Container("LBM_iteration", fIn.getBackend(), [desc, in, out, fl]() -> set::Launch {
            set::Launch l;
            l.signature = set::bytes_of(desc);
            l.run = [desc, in, out, fl](cudaStream_t s) { NEON_NGB_CHECK(ngb_bgrid_lbm_step(&desc, in, out, fl, s)); };
            return l;
        });
    }
}

// computeWallNghMask (LbmTools.h:327-376), in place on the packed flags.
template <int Q, typename FlagField>
auto computeWallNghMask(FlagField& flags) -> set::Container
{
    uint32_t* fl = flags.mem();
    if constexpr (std::is_same_v<typename FlagField::Grid, Neon::dGrid>) {
        const int32_3d d = flags.getDimension();
        return set::Container("LBM_wallMask", flags.getBackend(), [d, fl]() -> set::Launch {
            set::Launch l;
            l.signature = set::bytes_of(fl);
            l.run = [d, fl](cudaStream_t s) { NEON_NGB_CHECK(ngb_lbm_wall_mask(d.x, d.y, d.z, Q, fl, s)); };
            return l;
        });
    } else {
        const auto&    B = flags.getGrid().getBlocks();
        ngb_bgrid_desc desc{};
        desc.n_blocks = int32_t(B.nBlocks), desc.q = Q, desc.storage = NGB_STORE_F32;
        desc.origin = B.dOrigin, desc.mask = B.dMask, desc.conn = B.dConn;
        return set::Container("LBM_wallMask", flags.getBackend(), [desc, fl]() -> set::Launch {
            set::Launch l;
            l.signature = set::bytes_of(fl);
            l.run = [desc, fl](cudaStream_t s) { NEON_NGB_CHECK(ngb_bgrid_wall_mask(&desc, fl, s)); };
            return l;
        });
    }
}

}  // namespace gb300
}  // namespace Neon
