// Neon::set::Container and Loader for one GPU (libNeonSet/include/Neon/set/Containter.h:20-167,
// container/Loader_imp.h:101-186).
//
// A container holds the user's loading lambda. Running it calls the loading
// lambda with a Loader (which hands out field partitions and enforces Neon's
// rule that a non-const field cannot be loaded for a STENCIL pattern), gets
// the per-cell compute lambda back and launches one generic kernel over the
// grid's span. `prepare()` separates the two halves so that a Skeleton can
// capture launches into a CUDA graph and detect when the compute lambda's
// captured state changed (then it re-captures).
//
// Data views (one partition): a grid container runs over the STANDARD span
// (every cell), the INTERNAL span or the BOUNDARY span (dGrid: the z slabs of
// the stencil's radius at both ends; bGrid: empty, every block of a single
// partition is internal). A container made by the library around one ABI
// call (the LBM step, the Laplacian, ...) covers the whole grid when asked
// for INTERNAL and does nothing for BOUNDARY, so INTERNAL then BOUNDARY still
// visits every cell once.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

#include "Neon/core/core.h"
#include "Neon/set/Backend.h"

namespace Neon {
namespace set {

class Loader {
   public:
    explicit Loader(Execution exec = Execution::device) : mExecution(exec) {}

    // Non-const field: MAP access only (Loader_imp.h:115-121).
    template <typename Field_ta>
    auto load(Field_ta& field, Pattern pattern = Pattern::MAP, StencilSemantic = StencilSemantic::standard)
        -> std::enable_if_t<!std::is_const_v<Field_ta>, typename Field_ta::Partition&>
    {
        if (pattern == Pattern::STENCIL) {
            NeonException e("Loader");
            e << "Loading a non const field for a stencil operation is not supported in Neon";
            NEON_THROW(e);
        }
        mPartitions.emplace_back(std::make_shared<Holder<typename Field_ta::Partition>>(field.getPartition(mExecution)));
        return static_cast<Holder<typename Field_ta::Partition>*>(mPartitions.back().get())->p;
    }

    // Const field: any pattern.
    template <typename Field_ta>
    auto load(Field_ta& field, Pattern pattern = Pattern::MAP, StencilSemantic = StencilSemantic::standard)
        -> std::enable_if_t<std::is_const_v<Field_ta>, const typename Field_ta::Partition&>
    {
        if (pattern == Pattern::STENCIL) mStencil = true;
        mPartitions.emplace_back(std::make_shared<Holder<typename Field_ta::Partition>>(field.getPartition(mExecution)));
        return static_cast<Holder<typename Field_ta::Partition>*>(mPartitions.back().get())->p;
    }

    auto getExecution() const -> Execution { return mExecution; }
    // A field was loaded with the STENCIL pattern (the container reads neighbours).
    auto isStencil() const -> bool { return mStencil; }

   private:
    struct HolderBase {
        virtual ~HolderBase() = default;
    };
    template <typename P>
    struct Holder : HolderBase {
        explicit Holder(const P& x) : p(x) {}
        P p;
    };
    Execution                                mExecution;
    bool                                     mStencil = false;
    std::vector<std::shared_ptr<HolderBase>> mPartitions;
};

// One prepared launch: the kernel launch over the whole grid, optionally the
// launch over one data view, whether the container is a stencil, and the bytes
// of its parameters.
struct Launch {
    std::function<void(cudaStream_t)>           run;
    std::function<void(cudaStream_t, DataView)> runView;
    bool                                        stencil = false;
    std::vector<char>                           signature;

    void launch(cudaStream_t s, DataView dv) const
    {
        if (runView)
            runView(s, dv);
        else if (dv != DataView::BOUNDARY)
            run(s);
    }
};

class Container {
   public:
    Container() = default;
    Container(std::string name, Backend bk, std::function<Launch()> prepare)
        : mName(std::move(name)), mBackend(std::move(bk)), mPrepare(std::move(prepare))
    {
    }
    auto getName() const -> const std::string& { return mName; }
    auto prepare() const -> Launch { return mPrepare(); }
    auto getBackend() const -> const Backend& { return mBackend; }

    // Launch over data view `dv` on the backend's stream `streamIdx` (asynchronous).
    void run(int streamIdx = Backend::mainStreamIdx, DataView dv = DataView::STANDARD) const
    {
        if (!mPrepare) return;
        const Launch l = mPrepare();
        l.launch(mBackend.stream(streamIdx), dv);
    }

   private:
    std::string             mName;
    Backend                 mBackend;
    std::function<Launch()> mPrepare;
};

template <typename T>
inline std::vector<char> bytes_of(const T& v)
{
    std::vector<char> b(sizeof(T));
    std::memcpy(b.data(), &v, sizeof(T));
    return b;
}

}  // namespace set
}  // namespace Neon
