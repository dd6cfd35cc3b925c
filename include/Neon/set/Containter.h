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
    auto load(Field_ta& field, Pattern = Pattern::MAP, StencilSemantic = StencilSemantic::standard)
        -> std::enable_if_t<std::is_const_v<Field_ta>, const typename Field_ta::Partition&>
    {
        mPartitions.emplace_back(std::make_shared<Holder<typename Field_ta::Partition>>(field.getPartition(mExecution)));
        return static_cast<Holder<typename Field_ta::Partition>*>(mPartitions.back().get())->p;
    }

    auto getExecution() const -> Execution { return mExecution; }

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
    std::vector<std::shared_ptr<HolderBase>> mPartitions;
};

// One prepared launch: the kernel launch itself and the bytes of its parameters.
struct Launch {
    std::function<void(cudaStream_t)> run;
    std::vector<char>                 signature;
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

    // Launch on the backend's stream `streamIdx` (asynchronous).
    void run(int streamIdx = Backend::mainStreamIdx, DataView = DataView::STANDARD) const
    {
        if (!mPrepare) return;
        Launch l = mPrepare();
        l.run(mBackend.stream(streamIdx));
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
