// Neon::skeleton::Skeleton for one GPU (libNeonSkeleton/include/Neon/skeleton/Skeleton.h:12-74).
//
// sequence() records the containers in order (one partition: the dependency
// graph of Neon's MultiXpuGraph is the sequence itself, no halo nodes). run()
// prepares every container (calls its loading lambda), and launches one CUDA
// graph holding all the kernels. The graph is captured on the first run and
// replayed while every container's kernel parameters stay byte-identical;
// when a loading lambda produced different parameters (a scalar captured by
// value changed, another field was loaded), the sequence is captured again and
// the executable graph updated. The graph .dot dump of Skeleton.h:43 is
// written only when the environment variable NEON_GB300_DOT is set.
//
// OCC (MultiXpuGraph::optimizations, multiGpuGraph.cpp:106-200): with any
// option other than Occ::none, a stencil container runs as its INTERNAL launch
// followed by its BOUNDARY launch (the split of optimizeStandardOCC). With one
// partition there is no halo transfer between the two, and the extended forms
// (which also split the map containers feeding a stencil) give the same
// launches as the standard one.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "Neon/core/core.h"
#include "Neon/set/Backend.h"
#include "Neon/set/Containter.h"

namespace Neon {
namespace skeleton {

enum class Occ { standard, extended, twoWayExtended, none };

struct Options {
    Options() = default;
    Options(Occ occ, set::TransferMode transfer) : mOcc(occ), mTransfer(transfer) {}
    auto occ() const -> Occ { return mOcc; }
    auto transferMode() const -> set::TransferMode { return mTransfer; }
    Occ               mOcc = Occ::none;
    set::TransferMode mTransfer = set::TransferMode::get;
};

class Skeleton {
   public:
    Skeleton() = default;
    explicit Skeleton(const Backend& bk) { setBackend(bk); }
    Skeleton(const Skeleton&) = delete;
    Skeleton& operator=(const Skeleton&) = delete;
    Skeleton(Skeleton&& o) noexcept { *this = std::move(o); }
    Skeleton& operator=(Skeleton&& o) noexcept
    {
        release();
        mBackend = o.mBackend;
        mOps = std::move(o.mOps);
        mName = std::move(o.mName);
        mOptions = o.mOptions;
        mInited = o.mInited;
        mExec = o.mExec;
        mSignature = std::move(o.mSignature);
        o.mExec = nullptr;
        return *this;
    }
    ~Skeleton() { release(); }

    void setBackend(const Backend& bk)
    {
        mBackend = bk;
        mInited = true;
    }

    void sequence(const std::vector<set::Container>& operations, std::string name, Options options = Options())
    {
        if (!mInited) {
            NeonException e("Skeleton");
            e << "A backend was not set";
            NEON_THROW(e);
        }
        release();
        mOps = operations;
        mName = std::move(name);
        mOptions = options;
        mSignature.clear();
        if (std::getenv("NEON_GB300_DOT")) ioToDot(mName, mName);
    }

    void run(int streamIdx = Backend::mainStreamIdx)
    {
        std::vector<set::Launch> launches;
        launches.reserve(mOps.size());
        std::vector<char> sig;
        for (auto& op : mOps) {
            launches.push_back(op.prepare());
            sig.insert(sig.end(), launches.back().signature.begin(), launches.back().signature.end());
        }
        cudaStream_t s = mBackend.stream(streamIdx);
        // the "Skeleton" range of Skeleton.h:56-65, around the graph launch
        nvtxRangePushA("Skeleton");
        if (!mExec || sig != mSignature) capture(launches);
        mSignature = std::move(sig);
        const cudaError_t e = cudaGraphLaunch(mExec, s);
        nvtxRangePop();
        NEON_CUDA_CHECK(e);
    }

    void ioToDot(const std::string& fname, const std::string& graphname = "", bool = false) const
    {
        std::ofstream f(fname + ".dot");
        f << "digraph \"" << graphname << "\" {\n";
        for (size_t i = 0; i < mOps.size(); i++) {
            f << "  n" << i << " [label=\"" << mOps[i].getName() << "\"];\n";
            if (i) f << "  n" << i - 1 << " -> n" << i << ";\n";
        }
        f << "}\n";
    }

   private:
    void capture(std::vector<set::Launch>& launches)
    {
        cudaStream_t cs;
        NEON_CUDA_CHECK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        NEON_CUDA_CHECK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        try {
            for (auto& l : launches) {
                if (mOptions.occ() != Occ::none && l.stencil && l.runView) {
                    l.runView(cs, DataView::INTERNAL);
                    l.runView(cs, DataView::BOUNDARY);
                } else {
                    l.launch(cs, DataView::STANDARD);
                }
            }
        } catch (...) {
            cudaStreamEndCapture(cs, &g);
            if (g) cudaGraphDestroy(g);
            cudaStreamDestroy(cs);
            throw;
        }
        NEON_CUDA_CHECK(cudaStreamEndCapture(cs, &g));
        cudaStreamDestroy(cs);
        bool updated = false;
        if (mExec) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(mExec, g, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(mExec);
                mExec = nullptr;
            }
        }
        if (!updated) NEON_CUDA_CHECK(cudaGraphInstantiate(&mExec, g, 0));
        cudaGraphDestroy(g);
    }
    void release()
    {
        if (mExec) cudaGraphExecDestroy(mExec);
        mExec = nullptr;
    }

    Backend                     mBackend;
    std::vector<set::Container> mOps;
    std::string                 mName;
    Options                     mOptions;
    bool                        mInited = false;
    cudaGraphExec_t             mExec = nullptr;
    std::vector<char>           mSignature;
};

}  // namespace skeleton
}  // namespace Neon
