// Neon::eGrid (element-sparse grid) for one partition on one GPU
// (libNeonDomain/include/Neon/domain/details/eGrid/{eGrid_imp.h:8-129,
// ePartition_imp.h, eSpan_imp.h, eField_imp.h}).
//
// Construction evaluates the active-cell lambda on the host into a byte map
// and builds the element order, global mapping and stencil connectivity on the
// device (ngb_egrid_count / ngb_egrid_fill; one partition: the active cells in
// z, y, x order). Field layout SoA over elements: e + c * count. Neighbours go
// through the connectivity (conn[s * count + e], negative = none) with the
// stencil's 3-D offsets mapped to point indices by a (2r+1)^3 table
// (Partitioner1D.h:295-336: -33 for offsets outside the stencil).
// Containers launch one thread per element in 256-thread CTAs
// (eGrid_imp.h:25: default block 256 x 1 x 1).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "Neon/core/core.h"
#include "Neon/domain/Stencil.h"
#include "Neon/domain/interface.h"
#include "Neon/set/Backend.h"
#include "Neon/set/Containter.h"
#include "neon_gb300.h"

namespace Neon {
namespace domain {
namespace details {
namespace eGrid {

struct eIndex {
    int32_t mIdx = 0;
    eIndex() = default;
    NEON_CUDA_HOST_DEVICE explicit eIndex(int32_t i) : mIdx(i) {}
    NEON_CUDA_HOST_DEVICE int32_t helpGet() const { return mIdx; }
};

// Elements [firstOffset, firstOffset + count) (eSpan_imp.h). One partition:
// STANDARD and INTERNAL hold every element, BOUNDARY none.
struct eSpan {
    int32_t count = 0;
    int32_t firstOffset = 0;
    NEON_CUDA_HOST_DEVICE bool setAndValidate(eIndex& idx, int x) const
    {
        idx = eIndex(x + firstOffset);
        return x < count;
    }
};

template <typename T, int C = 0>
struct ePartition {
    using Type = T;
    using Idx = eIndex;
    using NghIdx = int8_t;
    using NghData = Neon::domain::NghData<T>;

    T*             mMem = nullptr;
    int            mCard = 1;
    int32_t        mCount = 0;        // elements allocated (the SoA pitch)
    const int32_t* mConn = nullptr;   // conn[s * count + e]
    const int32_t* mOrigin = nullptr; // 3 per element
    const int8_t*  mTable = nullptr;  // (2r+1)^3 offset -> stencil point
    int            mRadius = 0;

    NEON_CUDA_HOST_DEVICE int cardinality() const { return mCard; }
    NEON_CUDA_HOST_DEVICE T&  operator()(const eIndex& i, int c) const { return mMem[size_t(i.mIdx) + size_t(c) * size_t(mCount)]; }
    NEON_CUDA_HOST_DEVICE int32_3d getGlobalIndex(const eIndex& i) const
    {
        const int32_t* o = mOrigin + 3 * size_t(i.mIdx);
        return int32_3d(o[0], o[1], o[2]);
    }
    NEON_CUDA_HOST_DEVICE T* mem() const { return mMem; }
    // isValidNgh: the connectivity entry of point s, negative = no neighbour
    NEON_CUDA_HOST_DEVICE bool isValidNgh(const eIndex& i, NghIdx s, eIndex& out) const
    {
        if (s < 0) return false;  // offset outside the stencil
        out.mIdx = mConn[size_t(s) * size_t(mCount) + size_t(i.mIdx)];
        return out.mIdx > -1;
    }
    NEON_CUDA_HOST_DEVICE NghIdx pointOf(int dx, int dy, int dz) const
    {
        if (dx < -mRadius || dx > mRadius || dy < -mRadius || dy > mRadius || dz < -mRadius || dz > mRadius) return -1;
        const int p = 2 * mRadius + 1;
        return mTable[(dx + mRadius) + (dy + mRadius) * p + (dz + mRadius) * p * p];
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const eIndex& i, NghIdx s, int c) const
    {
        eIndex n;
        if (!isValidNgh(i, s, n)) return NghData(T{}, false);
        return NghData((*this)(n, c), true);
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const eIndex& i, const int8_3d& o, int c) const
    {
        return getNghData(i, pointOf(o.x, o.y, o.z), c);
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const eIndex& i, const int8_3d& o, int c, const T& alternative) const
    {
        NghData r = getNghData(i, pointOf(o.x, o.y, o.z), c);
        if (!r.isValid()) r.set(alternative, false);
        return r;
    }
    template <int dx, int dy, int dz>
    NEON_CUDA_HOST_DEVICE NghData getNghData(const eIndex& i, int c) const
    {
        return getNghData(i, pointOf(dx, dy, dz), c);
    }
    template <int dx, int dy, int dz>
    NEON_CUDA_HOST_DEVICE NghData getNghData(const eIndex& i, int c, const T& alternative) const
    {
        NghData r = getNghData(i, pointOf(dx, dy, dz), c);
        if (!r.isValid()) r.set(alternative, false);
        return r;
    }
};

#if defined(__CUDACC__)
template <typename F>
__global__ void __launch_bounds__(256) egrid_container_kernel(eSpan span, F f)
{
    eIndex idx;
    if (span.setAndValidate(idx, int(blockIdx.x * blockDim.x + threadIdx.x))) f(idx);
}
#endif

class eGrid;

// Shared element structure of an eGrid (device arrays + host copies).
struct ElementData {
    Backend              bk;
    int32_3d             dim;
    int32_t              count = 0;
    int                  radius = 0;
    int32_t*             dOrigin = nullptr;
    int32_t*             dConn = nullptr;
    int8_t*              dTable = nullptr;
    std::vector<int32_t> hOrigin;
    std::vector<int32_t> hConn;
    std::vector<int8_t>  hTable;
    ~ElementData()
    {
        if (dOrigin) cudaFree(dOrigin);
        if (dConn) cudaFree(dConn);
        if (dTable) cudaFree(dTable);
    }
};

template <typename T, int C = 0>
class eField {
   public:
    using Type = T;
    using Grid = eGrid;
    using Partition = ePartition<T, C>;
    using Idx = eIndex;
    static constexpr int Cardinality = C;

    eField() = default;
    eField(const std::string& name, std::shared_ptr<ElementData> elems, int card, T outside)
    {
        mData = std::make_shared<Data>();
        mData->name = name;
        mData->elems = elems;
        mData->card = card;
        const size_t n = size_t(elems->count) * card;
        mData->host.assign(n, outside);
        elems->bk.setDevice();
        NEON_CUDA_CHECK(cudaMalloc(&mData->dev, std::max<size_t>(n, 1) * sizeof(T)));
        NEON_CUDA_CHECK(cudaMemcpy(mData->dev, mData->host.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    }
    auto getPartition(Execution exec = Execution::device, int = 0, DataView = DataView::STANDARD) const -> Partition
    {
        const ElementData& E = *mData->elems;
        const bool         d = exec == Execution::device;
        Partition          p;
        p.mMem = d ? mData->dev : const_cast<T*>(mData->host.data());
        p.mCard = mData->card;
        p.mCount = E.count;
        p.mConn = d ? E.dConn : E.hConn.data();
        p.mOrigin = d ? E.dOrigin : E.hOrigin.data();
        p.mTable = d ? E.dTable : E.hTable.data();
        p.mRadius = E.radius;
        return p;
    }
    auto getGrid() const -> const Grid& { return *mData->grid; }
    auto getBackend() const -> const Backend& { return mData->elems->bk; }
    auto getName() const -> const std::string& { return mData->name; }
    auto cardinality() const -> int { return mData->card; }
    auto getUid() const -> uintptr_t { return reinterpret_cast<uintptr_t>(mData.get()); }
    auto mem() const -> T* { return mData->dev; }
    auto hostMem() const -> T* { return const_cast<T*>(mData->host.data()); }

    // Host loop over the elements in element order.
    template <typename L>
    void forEachActiveCell(L&& fn, computeMode_t = computeMode_t::par)
    {
        const ElementData& E = *mData->elems;
        for (int32_t e = 0; e < E.count; e++) {
            const index_3d g(E.hOrigin[3 * size_t(e)], E.hOrigin[3 * size_t(e) + 1], E.hOrigin[3 * size_t(e) + 2]);
            for (int c = 0; c < mData->card; c++) fn(g, c, mData->host[size_t(e) + size_t(c) * size_t(E.count)]);
        }
    }
    void updateDeviceData(int streamIdx = Backend::mainStreamIdx)
    {
        NEON_CUDA_CHECK(cudaMemcpyAsync(mData->dev, mData->host.data(), mData->host.size() * sizeof(T), cudaMemcpyHostToDevice,
                                        mData->elems->bk.stream(streamIdx)));
    }
    void updateHostData(int streamIdx = Backend::mainStreamIdx)
    {
        NEON_CUDA_CHECK(cudaMemcpyAsync(mData->host.data(), mData->dev, mData->host.size() * sizeof(T), cudaMemcpyDeviceToHost,
                                        mData->elems->bk.stream(streamIdx)));
    }
    auto newHaloUpdate(set::StencilSemantic, set::TransferMode, Execution) const -> set::Container { return set::Container(); }
    void setGrid(const Grid& g) { mData->grid = std::make_shared<Grid>(g); }

   private:
    struct Data {
        std::string                  name;
        std::shared_ptr<ElementData> elems;
        int                          card = 1;
        T*                           dev = nullptr;
        std::vector<T>               host;
        std::shared_ptr<const Grid>  grid;
        ~Data()
        {
            if (dev) cudaFree(dev);
        }
    };
    std::shared_ptr<Data> mData;
};

class eGrid {
   public:
    using Idx = eIndex;
    using Span = eSpan;
    template <typename T, int C = 0>
    using Field = eField<T, C>;
    template <typename T, int C = 0>
    using Partition = ePartition<T, C>;

    eGrid() = default;
    template <typename ActiveCellLambda>
    eGrid(const Backend& bk, const int32_3d& dim, const ActiveCellLambda& active, const Stencil& stencil,
          const double_3d& = double_3d(1, 1, 1), const double_3d& = double_3d(0, 0, 0))
    {
        mStencil = stencil;
        mElems = std::make_shared<ElementData>();
        auto& E = *mElems;
        E.bk = bk;
        E.dim = dim;
        bk.setDevice();
        // the active-cell lambda on the host (eGrid_imp.h:29-36), as a byte map
        const size_t         V = size_t(dim.rMul());
        std::vector<uint8_t> map(V);
        for (int z = 0; z < dim.z; z++)
            for (int y = 0; y < dim.y; y++)
                for (int x = 0; x < dim.x; x++)
                    map[size_t(x) + size_t(dim.x) * (size_t(y) + size_t(dim.y) * z)] = active(index_3d(x, y, z)) ? 1 : 0;
        // stencil points in the stencil's order, and the offset -> point table
        const auto&         pts = stencil.neighbours();
        std::vector<int8_t> points;
        for (const auto& p : pts) points.insert(points.end(), {int8_t(p.x), int8_t(p.y), int8_t(p.z)});
        E.radius = stencil.getRadius();
        const int p1 = 2 * E.radius + 1;
        E.hTable.assign(size_t(p1) * p1 * p1, int8_t(-33));
        for (size_t s = 0; s < pts.size(); s++)
            E.hTable[(pts[s].x + E.radius) + (pts[s].y + E.radius) * p1 + (pts[s].z + E.radius) * p1 * p1] = int8_t(s);
        // element order, global mapping and connectivity on the device
        uint8_t*     dmap = nullptr;
        int32_t*     elemOf = nullptr;
        int32_t*     scratch = nullptr;
        int32_t*     dn = nullptr;
        cudaStream_t s = bk.stream();
        NEON_CUDA_CHECK(cudaMalloc(&dmap, std::max<size_t>(V, 1)));
        NEON_CUDA_CHECK(cudaMalloc(&elemOf, std::max<size_t>(V, 1) * sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&scratch, size_t(NGB_EGRID_SCRATCH(dim.x, dim.y, dim.z)) * sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&dn, sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMemcpyAsync(dmap, map.data(), V, cudaMemcpyHostToDevice, s));
        NEON_NGB_CHECK(ngb_egrid_count(dim.x, dim.y, dim.z, dmap, elemOf, scratch, dn, s));
        NEON_CUDA_CHECK(cudaMemcpyAsync(&E.count, dn, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaStreamSynchronize(s));
        const size_t n = std::max<int32_t>(E.count, 1), np = std::max<size_t>(pts.size(), 1);
        NEON_CUDA_CHECK(cudaMalloc(&E.dOrigin, n * 3 * sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&E.dConn, n * np * sizeof(int32_t)));
        NEON_CUDA_CHECK(cudaMalloc(&E.dTable, E.hTable.size()));
        NEON_CUDA_CHECK(cudaMemcpyAsync(E.dTable, E.hTable.data(), E.hTable.size(), cudaMemcpyHostToDevice, s));
        NEON_NGB_CHECK(ngb_egrid_fill(dim.x, dim.y, dim.z, elemOf, E.count, points.data(), int32_t(pts.size()), E.dOrigin, E.dConn, s));
        E.hOrigin.resize(n * 3);
        E.hConn.resize(n * np);
        NEON_CUDA_CHECK(cudaMemcpyAsync(E.hOrigin.data(), E.dOrigin, n * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaMemcpyAsync(E.hConn.data(), E.dConn, n * np * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        NEON_CUDA_CHECK(cudaStreamSynchronize(s));
        cudaFree(dmap);
        cudaFree(elemOf);
        cudaFree(scratch);
        cudaFree(dn);
    }
    template <typename ActiveCellLambda>
    eGrid(const Backend& bk, const int32_3d& dim, const ActiveCellLambda& l, const std::vector<index_3d>& stencil,
          const double_3d& spacing = double_3d(1, 1, 1), const double_3d& origin = double_3d(0, 0, 0))
        : eGrid(bk, dim, l, Stencil(stencil), spacing, origin)
    {
    }

    auto getDimension() const -> int32_3d { return mElems->dim; }
    auto getBackend() const -> const Backend& { return mElems->bk; }
    auto getStencil() const -> const Stencil& { return mStencil; }
    auto getImplementationName() const -> std::string { return "eGrid"; }
    auto getNumActiveCells() const -> int64_t { return mElems->count; }
    auto toString() const -> std::string
    {
        return "[eGrid] " + mElems->dim.to_string() + " elements " + std::to_string(mElems->count);
    }
    // One partition: STANDARD and INTERNAL hold every element, BOUNDARY none
    // (eGrid_imp.h:74-116 with an empty boundary class).
    auto getSpan(Execution = Execution::device, int = 0, DataView dv = DataView::STANDARD) const -> eSpan
    {
        return eSpan{dv == DataView::BOUNDARY ? 0 : mElems->count, 0};
    }

    template <typename T, int C = 0>
    auto newField(const std::string& name, int cardinality, T inactiveValue, DataUse = DataUse::HOST_DEVICE,
                  MemoryOptions = MemoryOptions()) const -> Field<T, C>
    {
        Field<T, C> f(name, mElems, cardinality, inactiveValue);
        f.setGrid(*this);
        return f;
    }

#if defined(__CUDACC__)
    template <Execution execution = Execution::device, typename LoadingLambda = void*>
    auto newContainer(const std::string& name, LoadingLambda lambda) const -> set::Container
    {
        const std::shared_ptr<ElementData> elems = mElems;
        return set::Container(name, mElems->bk, [elems, lambda]() -> set::Launch {
            set::Loader L(execution);
            auto        f = lambda(L);
            set::Launch l;
            l.signature = set::bytes_of(f);
            l.stencil = L.isStencil();
            const int32_t count = elems->count;
            if constexpr (execution == Execution::device) {
                l.runView = [count, f](cudaStream_t s, DataView dv) {
                    const eSpan span{dv == DataView::BOUNDARY ? 0 : count, 0};
                    if (span.count == 0) return;
                    egrid_container_kernel<<<unsigned((span.count + 255) / 256), 256, 0, s>>>(span, f);
                    NEON_CUDA_CHECK(cudaGetLastError());
                };
            } else {
                l.runView = [count, f](cudaStream_t s, DataView dv) mutable {
                    if (dv == DataView::BOUNDARY) return;
                    NEON_CUDA_CHECK(cudaStreamSynchronize(s));
                    const eSpan span{count, 0};
                    eIndex      idx;
                    for (int32_t e = 0; e < count; e++)
                        if (span.setAndValidate(idx, e)) f(idx);
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
    Stencil                      mStencil;
    std::shared_ptr<ElementData> mElems;
};

}  // namespace eGrid
}  // namespace details
}  // namespace domain

using eGrid = domain::details::eGrid::eGrid;

}  // namespace Neon
