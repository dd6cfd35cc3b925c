// Neon::bGrid (8x8x8 blocks) for one partition on one GPU
// (libNeonDomain/include/Neon/domain/details/bGrid/{bGrid_imp.h:19-246, bPartition_imp.h:95-405,
// bSpan_imp.h:6-38, bIndex.h:63-109}).
//
// Construction evaluates the active-cell lambda on the host into a byte map
// and builds block order, active masks and 27-connectivity on the device
// (ngb_bgrid_count / ngb_bgrid_fill; bit-exact to Neon's single-partition
// construction). Field layout per block SoA: ((b*card + c)*512 + x + 8y + 64z).
// Containers launch one 8x8x8 CUDA block per data block (bGrid_imp.h:231-245);
// inactive voxels are skipped (bSpan::setAndValidate).
#pragma once
#include <cuda_runtime.h>

#include "Neon/core/core.h"
#include "Neon/domain/Stencil.h"
#include "Neon/domain/interface.h"
#include "Neon/set/Backend.h"
#include "Neon/set/Containter.h"
#include "neon_gb300.h"

namespace Neon {
namespace domain {
namespace details {
namespace bGrid {

struct bIndex {
    uint32_t mDataBlockIdx = 0;
    int8_3d  mInDataBlockIdx;
    bIndex() = default;
    NEON_CUDA_HOST_DEVICE bIndex(uint32_t b, int8_t x, int8_t y, int8_t z) : mDataBlockIdx(b), mInDataBlockIdx(x, y, z) {}
    NEON_CUDA_HOST_DEVICE int voxel() const { return mInDataBlockIdx.x + 8 * mInDataBlockIdx.y + 64 * mInDataBlockIdx.z; }
};

NEON_CUDA_HOST_DEVICE inline bool mask_active(const uint32_t* mask, uint32_t b, int v)
{
    return (mask[size_t(b) * 16 + (v >> 5)] >> (v & 31)) & 1u;
}

struct bSpan {
    uint32_t        nBlocks = 0;
    const uint32_t* mask = nullptr;
    NEON_CUDA_HOST_DEVICE bool setAndValidate(bIndex& idx, uint32_t block, int x, int y, int z) const
    {
        idx = bIndex(block, int8_t(x), int8_t(y), int8_t(z));
        return block < nBlocks && mask_active(mask, block, idx.voxel());
    }
};

template <typename T, int C = 0>
struct bPartition {
    using Type = T;
    using Idx = bIndex;
    using NghIdx = int8_3d;
    using NghData = Neon::domain::NghData<T>;

    T*              mMem = nullptr;
    int             mCard = 1;
    const uint32_t* mMask = nullptr;
    const uint32_t* mConn = nullptr;
    const int32_t*  mOrigin = nullptr;

    NEON_CUDA_HOST_DEVICE int cardinality() const { return mCard; }
    NEON_CUDA_HOST_DEVICE T&  operator()(const bIndex& i, int c) const
    {
        return mMem[(size_t(i.mDataBlockIdx) * mCard + c) * 512 + i.voxel()];
    }
    NEON_CUDA_HOST_DEVICE int32_3d getGlobalIndex(const bIndex& i) const
    {
        const int32_t* o = mOrigin + 3 * size_t(i.mDataBlockIdx);
        return int32_3d(o[0] + i.mInDataBlockIdx.x, o[1] + i.mInDataBlockIdx.y, o[2] + i.mInDataBlockIdx.z);
    }
    // bPartition::helpGetNghIdx + helpNghPitch (bPartition_imp.h:109-309)
    NEON_CUDA_HOST_DEVICE bool nghIdx(const bIndex& i, int ox, int oy, int oz, bIndex& out) const
    {
        int       nx = i.mInDataBlockIdx.x + ox, ny = i.mInDataBlockIdx.y + oy, nz = i.mInDataBlockIdx.z + oz;
        const int fx = nx < 0 ? -1 : (nx >= 8 ? 1 : 0), fy = ny < 0 ? -1 : (ny >= 8 ? 1 : 0), fz = nz < 0 ? -1 : (nz >= 8 ? 1 : 0);
        uint32_t  b = i.mDataBlockIdx;
        if (fx | fy | fz) {
            nx -= 8 * fx, ny -= 8 * fy, nz -= 8 * fz;
            b = mConn[size_t(b) * 27 + (fx + 1) + 3 * (fy + 1) + 9 * (fz + 1)];
            if (b == NGB_BGRID_NO_BLOCK) return false;
        }
        out = bIndex(b, int8_t(nx), int8_t(ny), int8_t(nz));
        return mask_active(mMask, b, out.voxel());
    }
    template <int dx, int dy, int dz>
    NEON_CUDA_HOST_DEVICE NghData getNghData(const bIndex& i, int c) const
    {
        bIndex n;
        if (!nghIdx(i, dx, dy, dz, n)) return NghData(T{}, false);
        return NghData((*this)(n, c), true);
    }
    template <int dx, int dy, int dz>
    NEON_CUDA_HOST_DEVICE NghData getNghData(const bIndex& i, int c, const T& alternative) const
    {
        bIndex n;
        if (!nghIdx(i, dx, dy, dz, n)) return NghData(alternative, false);
        return NghData((*this)(n, c), true);
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const bIndex& i, const int8_3d& o, int c) const
    {
        bIndex n;
        if (!nghIdx(i, o.x, o.y, o.z, n)) return NghData(T{}, false);
        return NghData((*this)(n, c), true);
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const bIndex& i, const int8_3d& o, int c, const T& alternative) const
    {
        bIndex n;
        if (!nghIdx(i, o.x, o.y, o.z, n)) return NghData(alternative, false);
        return NghData((*this)(n, c), true);
    }
};

#if defined(__CUDACC__)
template <typename F>
__global__ void __launch_bounds__(512) bgrid_container_kernel(bSpan span, F f)
{
    bIndex idx;
    if (span.setAndValidate(idx, blockIdx.x, threadIdx.x, threadIdx.y, threadIdx.z)) f(idx);
}
#endif

class bGrid;

// Shared block structure of a bGrid (device arrays + host copies).
struct BlockData {
    Backend               bk;
    int32_3d              dim;
    uint32_t              nBlocks = 0;
    uint64_t              nActive = 0;
    int32_t*              dOrigin = nullptr;
    uint32_t*             dMask = nullptr;
    uint32_t*             dConn = nullptr;
    std::vector<int32_t>  hOrigin;
    std::vector<uint32_t> hMask;
    std::vector<uint32_t> hConn;
    ~BlockData()
    {
        if (dOrigin) cudaFree(dOrigin);
        if (dMask) cudaFree(dMask);
        if (dConn) cudaFree(dConn);
    }
};

template <typename T, int C = 0>
class bField {
   public:
    using Type = T;
    using Grid = bGrid;
    using Partition = bPartition<T, C>;
    using Idx = bIndex;
    static constexpr int Cardinality = C;

    bField() = default;
    bField(const std::string& name, std::shared_ptr<BlockData> blocks, int card, T outside)
    {
        mData = std::make_shared<Data>();
        mData->name = name;
        mData->blocks = blocks;
        mData->card = card;
        const size_t n = size_t(blocks->nBlocks) * card * 512;
        mData->host.assign(n, outside);
        blocks->bk.setDevice();
        NEON_CUDA_CHECK(cudaMalloc(&mData->dev, std::max<size_t>(n, 1) * sizeof(T)));
        NEON_CUDA_CHECK(cudaMemcpy(mData->dev, mData->host.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    }
    auto getPartition(Execution exec = Execution::device, int = 0, DataView = DataView::STANDARD) const -> Partition
    {
        Partition p;
        p.mMem = exec == Execution::device ? mData->dev : const_cast<T*>(mData->host.data());
        p.mCard = mData->card;
        p.mMask = exec == Execution::device ? mData->blocks->dMask : mData->blocks->hMask.data();
        p.mConn = exec == Execution::device ? mData->blocks->dConn : mData->blocks->hConn.data();
        p.mOrigin = exec == Execution::device ? mData->blocks->dOrigin : mData->blocks->hOrigin.data();
        return p;
    }
    auto getGrid() const -> const Grid& { return *mData->grid; }
    auto getBackend() const -> const Backend& { return mData->blocks->bk; }
    auto getName() const -> const std::string& { return mData->name; }
    auto cardinality() const -> int { return mData->card; }
    auto getUid() const -> uintptr_t { return reinterpret_cast<uintptr_t>(mData.get()); }
    auto mem() const -> T* { return mData->dev; }
    auto hostMem() const -> T* { return const_cast<T*>(mData->host.data()); }

    // Host loop over active voxels, block order then x fastest in the block.
    template <typename L>
    void forEachActiveCell(L&& fn, computeMode_t = computeMode_t::par)
    {
        const auto& B = *mData->blocks;
        for (uint32_t b = 0; b < B.nBlocks; b++)
            for (int v = 0; v < 512; v++) {
                if (!mask_active(B.hMask.data(), b, v)) continue;
                const index_3d g(B.hOrigin[3 * b] + (v & 7), B.hOrigin[3 * b + 1] + ((v >> 3) & 7), B.hOrigin[3 * b + 2] + (v >> 6));
                for (int c = 0; c < mData->card; c++) fn(g, c, mData->host[(size_t(b) * mData->card + c) * 512 + v]);
            }
    }
    void updateDeviceData(int streamIdx = Backend::mainStreamIdx)
    {
        NEON_CUDA_CHECK(cudaMemcpyAsync(mData->dev, mData->host.data(), mData->host.size() * sizeof(T), cudaMemcpyHostToDevice,
                                        mData->blocks->bk.stream(streamIdx)));
    }
    void updateHostData(int streamIdx = Backend::mainStreamIdx)
    {
        NEON_CUDA_CHECK(cudaMemcpyAsync(mData->host.data(), mData->dev, mData->host.size() * sizeof(T), cudaMemcpyDeviceToHost,
                                        mData->blocks->bk.stream(streamIdx)));
    }
    auto newHaloUpdate(set::StencilSemantic, set::TransferMode, Execution) const -> set::Container { return set::Container(); }
    void setGrid(const Grid& g) { mData->grid = std::make_shared<Grid>(g); }

   private:
    struct Data {
        std::string                 name;
        std::shared_ptr<BlockData>  blocks;
        int                         card = 1;
        T*                          dev = nullptr;
        std::vector<T>              host;
        std::shared_ptr<const Grid> grid;
        ~Data()
        {
            if (dev) cudaFree(dev);
        }
    };
    std::shared_ptr<Data> mData;
};

class bGrid {
   public:
    using Idx = bIndex;
    using Span = bSpan;
    template <typename T, int C = 0>
    using Field = bField<T, C>;
    template <typename T, int C = 0>
    using Partition = bPartition<T, C>;

    bGrid() = default;
    template <typename ActiveCellLambda>
    bGrid(const Backend& bk, const int32_3d& dim, const ActiveCellLambda& active, const Stencil& stencil,
          const double_3d& = double_3d(1, 1, 1), const double_3d& = double_3d(0, 0, 0))
    {
        mStencil = stencil;
        mBlocks = std::make_shared<BlockData>();
        auto& B = *mBlocks;
        B.bk = bk;
        B.dim = dim;
        bk.setDevice();
        // the active-cell lambda on the host (bGrid_imp.h:80-136), as a byte map
        const size_t         V = size_t(dim.rMul());
        std::vector<uint8_t> map(V);
        for (int z = 0; z < dim.z; z++)
            for (int y = 0; y < dim.y; y++)
                for (int x = 0; x < dim.x; x++)
                    map[size_t(x) + size_t(dim.x) * (size_t(y) + size_t(dim.y) * z)] = active(index_3d(x, y, z)) ? 1 : 0;
        const size_t ncand = size_t(NGB_BGRID_BLOCKS(dim.x)) * NGB_BGRID_BLOCKS(dim.y) * NGB_BGRID_BLOCKS(dim.z);
        uint8_t*     dmap = nullptr;
        int32_t*     blockOf = nullptr;
        uint32_t*    dn = nullptr;
        unsigned long long* dact = nullptr;
        cudaStream_t s = bk.stream();
        NEON_CUDA_CHECK(cudaMalloc(&dmap, std::max<size_t>(V, 1)));
        NEON_CUDA_CHECK(cudaMalloc(&blockOf, std::max<size_t>(ncand, 1) * sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&dn, sizeof(uint32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&dact, sizeof(unsigned long long)));
        NEON_CUDA_CHECK(cudaMemcpyAsync(dmap, map.data(), V, cudaMemcpyHostToDevice, s));
        NEON_NGB_CHECK(ngb_bgrid_count(dim.x, dim.y, dim.z, dmap, blockOf, dn, s));
        NEON_CUDA_CHECK(cudaMemcpyAsync(&B.nBlocks, dn, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaStreamSynchronize(s));
        const size_t nb = std::max<uint32_t>(B.nBlocks, 1);
        NEON_CUDA_CHECK(cudaMalloc(&B.dOrigin, nb * 3 * sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&B.dMask, nb * 16 * sizeof(uint32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&B.dConn, nb * 27 * sizeof(uint32_t)));
        NEON_NGB_CHECK(ngb_bgrid_fill(dim.x, dim.y, dim.z, dmap, blockOf, B.dOrigin, B.dMask, B.dConn, dact, s));
        B.hOrigin.resize(nb * 3);
        B.hMask.resize(nb * 16);
        B.hConn.resize(nb * 27);
        NEON_CUDA_CHECK(cudaMemcpyAsync(B.hOrigin.data(), B.dOrigin, nb * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaMemcpyAsync(B.hMask.data(), B.dMask, nb * 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaMemcpyAsync(B.hConn.data(), B.dConn, nb * 27 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaMemcpyAsync(&B.nActive, dact, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaStreamSynchronize(s));
        cudaFree(dmap);
        cudaFree(blockOf);
        cudaFree(dn);
        cudaFree(dact);
    }
    template <typename ActiveCellLambda>
    bGrid(const Backend& bk, const int32_3d& dim, const ActiveCellLambda& l, const std::vector<index_3d>& stencil,
          const double_3d& spacing = double_3d(1, 1, 1), const double_3d& origin = double_3d(0, 0, 0))
        : bGrid(bk, dim, l, Stencil(stencil), spacing, origin)
    {
    }

    auto getDimension() const -> int32_3d { return mBlocks->dim; }
    auto getBackend() const -> const Backend& { return mBlocks->bk; }
    auto getImplementationName() const -> std::string { return "bGrid"; }
    auto getNumBlocks() const -> uint32_t { return mBlocks->nBlocks; }
    auto getNumActiveCells() const -> uint64_t { return mBlocks->nActive; }
    auto getBlocks() const -> const BlockData& { return *mBlocks; }
    auto toString() const -> std::string
    {
        return "[bGrid] " + mBlocks->dim.to_string() + " blocks " + std::to_string(mBlocks->nBlocks);
    }
    // One partition: STANDARD and INTERNAL hold every active block, BOUNDARY none
    // (a single partition's blocks are all internal, bGrid_imp.h:57).
    auto getSpan(Execution = Execution::device, int = 0, DataView dv = DataView::STANDARD) const -> bSpan
    {
        if (dv == DataView::BOUNDARY) return bSpan{0, mBlocks->dMask};
        return bSpan{mBlocks->nBlocks, mBlocks->dMask};
    }

    template <typename T, int C = 0>
    auto newField(const std::string& name, int cardinality, T inactiveValue, DataUse = DataUse::HOST_DEVICE,
                  MemoryOptions = MemoryOptions()) const -> Field<T, C>
    {
        Field<T, C> f(name, mBlocks, cardinality, inactiveValue);
        f.setGrid(*this);
        return f;
    }

#if defined(__CUDACC__)
    template <Execution execution = Execution::device, typename LoadingLambda = void*>
    auto newContainer(const std::string& name, LoadingLambda lambda) const -> set::Container
    {
        const bSpan                      span = getSpan();
        const std::shared_ptr<BlockData> blocks = mBlocks;
        return set::Container(name, mBlocks->bk, [span, blocks, lambda]() -> set::Launch {
            set::Loader L(execution);
            auto        f = lambda(L);
            set::Launch l;
            l.signature = set::bytes_of(f);
            l.stencil = L.isStencil();
            // one partition: every block is internal, the BOUNDARY view is empty
            if constexpr (execution == Execution::device) {
                l.runView = [span, f](cudaStream_t s, DataView dv) {
                    if (span.nBlocks == 0 || dv == DataView::BOUNDARY) return;
                    bgrid_container_kernel<<<span.nBlocks, dim3(8, 8, 8), 0, s>>>(span, f);
                    NEON_CUDA_CHECK(cudaGetLastError());
                };
            } else {
                l.runView = [blocks, f](cudaStream_t s, DataView dv) mutable {
                    if (dv == DataView::BOUNDARY) return;
                    NEON_CUDA_CHECK(cudaStreamSynchronize(s));
                    const bSpan hs{blocks->nBlocks, blocks->hMask.data()};
                    bIndex      idx;
                    for (uint32_t b = 0; b < blocks->nBlocks; b++)
                        for (int v = 0; v < 512; v++)
                            if (hs.setAndValidate(idx, b, v & 7, (v >> 3) & 7, v >> 6)) f(idx);
                };
            }
            l.run = [rv = l.runView](cudaStream_t s) { rv(s, DataView::STANDARD); };
            return l;
        });
    }
    template <Execution execution = Execution::device, typename LoadingLambda = void*>
    auto newContainer(const std::string& name, index_3d, size_t, LoadingLambda lambda) const -> set::Container
    {
        return newContainer<execution>(name, lambda);
    }
#endif

   private:
    std::shared_ptr<BlockData> mBlocks;
    Stencil                    mStencil;
};

}  // namespace bGrid
}  // namespace details
}  // namespace domain

using bGrid = domain::details::bGrid::bGrid;

}  // namespace Neon
