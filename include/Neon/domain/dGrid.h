// Neon::dGrid for one partition on one GPU
// (libNeonDomain/include/Neon/domain/details/dGrid/{dGrid.h:41-232, dField_imp.h, dPartition.h:19-392}).
//
// Field layout: element (x, y, z, c) at x + nx*(y + ny*z) + c*nx*ny*nz (SoA,
// dField_imp.h:71-87). Neighbour validity: inside [0, dim) (dPartition.h:228-263).
// Containers launch one thread per cell with 256x1x1 blocks (dGrid_imp.h:16).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "Neon/core/core.h"
#include "Neon/domain/Stencil.h"
#include "Neon/domain/interface.h"
#include "Neon/set/Backend.h"
#include "Neon/set/Containter.h"
#include "neon_gb300.h"

namespace Neon {
namespace domain {
namespace details {
namespace dGrid {

struct dIndex {
    int32_3d mLocation;
    dIndex() = default;
    NEON_CUDA_HOST_DEVICE dIndex(int x, int y, int z) : mLocation(x, y, z) {}
    NEON_CUDA_HOST_DEVICE auto get() const -> const int32_3d& { return mLocation; }
    NEON_CUDA_HOST_DEVICE auto getLocation() const -> const int32_3d& { return mLocation; }
};

// Cells of one data view (dSpan_imp.h:6-43, span table of dGrid_imp.h:79-128,
// one partition: no halo). `dim` is the view's extent; thread z maps to grid z
// by zOffset (INTERNAL: z + r over nz - 2r planes) or, for BOUNDARY, the lower
// r planes stay and the upper r go to nz - r .. nz - 1 (r = the stencil's z
// radius). The reference maps the upper boundary planes from the view's own
// extent (z + r - 1), which for one partition would revisit internal planes;
// here they are the grid's top r planes, so INTERNAL and BOUNDARY together
// cover every cell once.
struct dSpan {
    int32_3d dim;            // extent of the view
    int      zOffset = 0;    // INTERNAL: r
    int      zUpper = 0;     // BOUNDARY: first thread z of the upper slab (r), 0 otherwise
    int      zUpperShift = 0;  // BOUNDARY: nz - 2r
    NEON_CUDA_HOST_DEVICE bool setAndValidate(dIndex& idx, int x, int y, int z) const
    {
        const bool ok = x < dim.x && y < dim.y && z < dim.z;
        const int  gz = z + zOffset + ((zUpper > 0 && z >= zUpper) ? zUpperShift : 0);
        idx = dIndex(x, y, gz);
        return ok;
    }
};

// The span of data view `dv` of an nx x ny x nz partition whose stencil reaches
// r planes in z.
inline dSpan make_dspan(const int32_3d& d, int r, DataView dv)
{
    dSpan s;
    s.dim = d;
    if (dv == DataView::STANDARD || r <= 0) {
        if (dv == DataView::BOUNDARY) s.dim.z = 0;  // no stencil reach: nothing on the boundary
        return s;
    }
    const int rr = r < d.z ? r : d.z;
    if (dv == DataView::INTERNAL) {
        s.dim.z = d.z - 2 * rr > 0 ? d.z - 2 * rr : 0;
        s.zOffset = rr;
    } else {  // BOUNDARY: the lower and upper slabs (all of z when they meet)
        if (2 * rr >= d.z) return s;
        s.dim.z = 2 * rr;
        s.zUpper = rr;
        s.zUpperShift = d.z - 2 * rr;
    }
    return s;
}

template <typename T, int C = 0>
struct dPartition {
    using Type = T;
    using Idx = dIndex;
    using NghIdx = int8_3d;
    using NghData = Neon::domain::NghData<T>;

    T*       mMem = nullptr;
    int32_3d mDim;
    int      mCard = 1;
    int64_t  mPitchCard = 0;  // nx*ny*nz

    NEON_CUDA_HOST_DEVICE int     cardinality() const { return mCard; }
    NEON_CUDA_HOST_DEVICE int64_t pitch(const int32_3d& p, int c) const
    {
        return int64_t(p.x) + int64_t(mDim.x) * (int64_t(p.y) + int64_t(mDim.y) * p.z) + int64_t(c) * mPitchCard;
    }
    NEON_CUDA_HOST_DEVICE T&       operator()(const dIndex& i, int c) const { return mMem[pitch(i.mLocation, c)]; }
    NEON_CUDA_HOST_DEVICE int32_3d getGlobalIndex(const dIndex& i) const { return i.mLocation; }
    NEON_CUDA_HOST_DEVICE T*       mem() const { return mMem; }

    NEON_CUDA_HOST_DEVICE bool valid(const int32_3d& p) const
    {
        return p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < mDim.x && p.y < mDim.y && p.z < mDim.z;
    }
    template <int dx, int dy, int dz>
    NEON_CUDA_HOST_DEVICE NghData getNghData(const dIndex& i, int c) const
    {
        const int32_3d p(i.mLocation.x + dx, i.mLocation.y + dy, i.mLocation.z + dz);
        if (!valid(p)) return NghData(T{}, false);
        return NghData(mMem[pitch(p, c)], true);
    }
    template <int dx, int dy, int dz>
    NEON_CUDA_HOST_DEVICE NghData getNghData(const dIndex& i, int c, const T& alternative) const
    {
        const int32_3d p(i.mLocation.x + dx, i.mLocation.y + dy, i.mLocation.z + dz);
        if (!valid(p)) return NghData(alternative, false);
        return NghData(mMem[pitch(p, c)], true);
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const dIndex& i, const int8_3d& o, int c) const
    {
        const int32_3d p(i.mLocation.x + o.x, i.mLocation.y + o.y, i.mLocation.z + o.z);
        if (!valid(p)) return NghData(T{}, false);
        return NghData(mMem[pitch(p, c)], true);
    }
    NEON_CUDA_HOST_DEVICE NghData getNghData(const dIndex& i, const int8_3d& o, int c, const T& alternative) const
    {
        const int32_3d p(i.mLocation.x + o.x, i.mLocation.y + o.y, i.mLocation.z + o.z);
        if (!valid(p)) return NghData(alternative, false);
        return NghData(mMem[pitch(p, c)], true);
    }
};

#if defined(__CUDACC__)
template <typename F>
__global__ void __launch_bounds__(256) dgrid_container_kernel(dSpan span, F f)
{
    dIndex idx;
    if (span.setAndValidate(idx, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y, blockIdx.z)) f(idx);
}
#endif

class dGrid;

template <typename T, int C = 0>
class dField {
   public:
    using Type = T;
    using Grid = dGrid;
    using Partition = dPartition<T, C>;
    using Idx = dIndex;
    static constexpr int Cardinality = C;

    dField() = default;
    dField(const std::string& name, const Backend& bk, int32_3d dim, int card, T outside)
    {
        mData = std::make_shared<Data>();
        mData->name = name;
        mData->bk = bk;
        mData->dim = dim;
        mData->card = card;
        mData->outside = outside;
        const size_t n = size_t(dim.rMul()) * card;
        mData->host.assign(n, outside);
        bk.setDevice();
        NEON_CUDA_CHECK(cudaMalloc(&mData->dev, std::max<size_t>(n, 1) * sizeof(T)));
        NEON_CUDA_CHECK(cudaMemcpy(mData->dev, mData->host.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    }

    auto getPartition(Execution exec = Execution::device, int = 0, DataView = DataView::STANDARD) const -> Partition
    {
        Partition p;
        p.mMem = exec == Execution::device ? mData->dev : const_cast<T*>(mData->host.data());
        p.mDim = mData->dim;
        p.mCard = mData->card;
        p.mPitchCard = int64_t(mData->dim.rMul());
        return p;
    }
    auto getGrid() const -> const Grid& { return *mData->grid; }
    auto getBackend() const -> const Backend& { return mData->bk; }
    auto getName() const -> const std::string& { return mData->name; }
    auto cardinality() const -> int { return mData->card; }
    auto getDimension() const -> int32_3d { return mData->dim; }
    auto getUid() const -> uintptr_t { return reinterpret_cast<uintptr_t>(mData.get()); }
    // raw device pointer (the C-ABI boundary)
    auto mem() const -> T* { return mData->dev; }
    auto hostMem() const -> T* { return const_cast<T*>(mData->host.data()); }

    auto getReference(const index_3d& p, int c) -> T& { return mData->host[pitch(p, c)]; }
    auto operator()(const index_3d& p, int c) const -> T { return mData->host[pitch(p, c)]; }

    // Host loop over every cell (dense grid: every cell is active).
    template <typename L>
    void forEachActiveCell(L&& fn, computeMode_t = computeMode_t::par)
    {
        const int32_3d d = mData->dim;
        for (int c = 0; c < mData->card; c++)
            for (int z = 0; z < d.z; z++)
                for (int y = 0; y < d.y; y++)
                    for (int x = 0; x < d.x; x++) fn(index_3d(x, y, z), c, mData->host[pitch(index_3d(x, y, z), c)]);
    }
    void updateDeviceData(int streamIdx = Backend::mainStreamIdx)
    {
        NEON_CUDA_CHECK(cudaMemcpyAsync(mData->dev, mData->host.data(), mData->host.size() * sizeof(T), cudaMemcpyHostToDevice,
                                        mData->bk.stream(streamIdx)));
    }
    void updateHostData(int streamIdx = Backend::mainStreamIdx)
    {
        NEON_CUDA_CHECK(cudaMemcpyAsync(mData->host.data(), mData->dev, mData->host.size() * sizeof(T), cudaMemcpyDeviceToHost,
                                        mData->bk.stream(streamIdx)));
    }
    // One partition: nothing to exchange (dField_imp.h:546-641 is multi-device only).
    auto newHaloUpdate(set::StencilSemantic, set::TransferMode, Execution) const -> set::Container { return set::Container(); }

    void setGrid(const Grid& g) { mData->grid = std::make_shared<Grid>(g); }

   private:
    size_t pitch(const index_3d& p, int c) const
    {
        return size_t(p.x) + size_t(mData->dim.x) * (size_t(p.y) + size_t(mData->dim.y) * p.z) + size_t(c) * mData->dim.rMul();
    }
    struct Data {
        std::string    name;
        Backend        bk;
        int32_3d       dim;
        int            card = 1;
        T              outside{};
        T*             dev = nullptr;
        std::vector<T> host;
        std::shared_ptr<const Grid> grid;
        ~Data()
        {
            if (dev) cudaFree(dev);
        }
    };
    std::shared_ptr<Data> mData;
};

class dGrid {
   public:
    using Idx = dIndex;
    using Span = dSpan;
    template <typename T, int C = 0>
    using Field = dField<T, C>;
    template <typename T, int C = 0>
    using Partition = dPartition<T, C>;

    dGrid() = default;
    template <typename ActiveCellLambda>
    dGrid(const Backend& bk, const int32_3d& dimension, const ActiveCellLambda&, const Stencil& stencil,
          const double_3d& spacing = double_3d(1, 1, 1), const double_3d& origin = double_3d(0, 0, 0))
    {
        mData = std::make_shared<Data>();
        mData->bk = bk;
        mData->dim = dimension;
        mData->stencil = stencil;
        mData->spacing = spacing;
        mData->origin = origin;
    }
    template <typename ActiveCellLambda>
    dGrid(const Backend& bk, const int32_3d& dimension, const ActiveCellLambda& l, const std::vector<index_3d>& stencil,
          const double_3d& spacing = double_3d(1, 1, 1), const double_3d& origin = double_3d(0, 0, 0))
        : dGrid(bk, dimension, l, Stencil(stencil), spacing, origin)
    {
    }

    auto getDimension() const -> int32_3d { return mData->dim; }
    auto getBackend() const -> const Backend& { return mData->bk; }
    auto getStencil() const -> const Stencil& { return mData->stencil; }
    auto getImplementationName() const -> std::string { return "dGrid"; }
    auto getSpan(Execution = Execution::device, int = 0, DataView dv = DataView::STANDARD) const -> dSpan
    {
        return make_dspan(mData->dim, zRadius(), dv);
    }
    // Planes a stencil of this grid reaches in z (the halo radius of dGrid_imp.h:65-70).
    auto zRadius() const -> int
    {
        int r = 0;
        for (const auto& p : mData->stencil.neighbours()) r = std::max(r, std::abs(p.z));
        return r;
    }
    auto toString() const -> std::string { return "[dGrid] " + mData->dim.to_string(); }

    template <typename T, int C = 0>
    auto newField(const std::string& name, int cardinality, T inactiveValue, DataUse = DataUse::HOST_DEVICE,
                  MemoryOptions = MemoryOptions()) const -> Field<T, C>
    {
        Field<T, C> f(name, mData->bk, mData->dim, cardinality, inactiveValue);
        f.setGrid(*this);
        return f;
    }

#if defined(__CUDACC__)
    template <Execution execution = Execution::device, typename LoadingLambda = void*>
    auto newContainer(const std::string& name, LoadingLambda lambda) const -> set::Container
    {
        const int32_3d dim = mData->dim;
        const int      r = zRadius();
        const Backend  bk = mData->bk;
        return set::Container(name, bk, [dim, r, lambda]() -> set::Launch {
            set::Loader L(execution);
            auto        f = lambda(L);
            set::Launch l;
            l.signature = set::bytes_of(f);
            l.stencil = L.isStencil();
            if constexpr (execution == Execution::device) {
                l.runView = [dim, r, f](cudaStream_t s, DataView dv) {
                    const dSpan span = make_dspan(dim, r, dv);
                    if (span.dim.x <= 0 || span.dim.y <= 0 || span.dim.z <= 0) return;
                    const dim3 grid((span.dim.x + 255) / 256, span.dim.y, span.dim.z);
                    dgrid_container_kernel<<<grid, 256, 0, s>>>(span, f);
                    NEON_CUDA_CHECK(cudaGetLastError());
                };
            } else {
                l.runView = [dim, r, f](cudaStream_t s, DataView dv) mutable {
                    const dSpan span = make_dspan(dim, r, dv);
                    NEON_CUDA_CHECK(cudaStreamSynchronize(s));
                    dIndex idx;
                    for (int z = 0; z < span.dim.z; z++)
                        for (int y = 0; y < span.dim.y; y++)
                            for (int x = 0; x < span.dim.x; x++)
                                if (span.setAndValidate(idx, x, y, z)) f(idx);
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

    // Grid dot product into a PatternScalar (dGrid.h:148-169; FP64 accumulation on the device).
    template <typename T>
    auto dot(const std::string& name, const Field<T>& a, const Field<T>& b, PatternScalar<T>& scalar) const -> set::Container
    {
        const Backend bk = mData->bk;
        return set::Container(name, bk, [a, b, scalar]() mutable -> set::Launch {
            set::Launch l;
            const int64_t n = int64_t(a.getDimension().rMul()) * a.cardinality();
            l.signature = set::bytes_of(a.mem());
            l.run = [a, b, scalar, n](cudaStream_t s) mutable {
                scalar.ensureScratch(n);
                NEON_NGB_CHECK(ngb_dot(n, sizeof(T) == 8 ? NGB_STORE_F64 : NGB_STORE_F32, a.mem(), b.mem(), scalar.devPtr(),
                                       scalar.scratch(), s));
            };
            return l;
        });
    }
#endif
    template <typename T>
    auto newPatternScalar() const -> PatternScalar<T>
    {
        return PatternScalar<T>(mData->bk);
    }

   private:
    struct Data {
        Backend   bk;
        int32_3d  dim;
        Stencil   stencil;
        double_3d spacing, origin;
    };
    std::shared_ptr<Data> mData;
};

}  // namespace dGrid
}  // namespace details
}  // namespace domain

using dGrid = domain::details::dGrid::dGrid;

}  // namespace Neon
