// Neon::Backend for one GPU and one partition (libNeonSet/src/set/Backend.cpp:32-134).
// Streams are created on first use; index 0 is Backend::mainStreamIdx.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <vector>

#include "Neon/core/core.h"

namespace Neon {

#define NEON_CUDA_CHECK(expr)                                                             \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            ::Neon::NeonException ex_("CUDA");                                            \
            ex_ << #expr << ": " << cudaGetErrorString(e_) << " (" << __FILE__ << ":" << __LINE__ << ")"; \
            throw ex_;                                                                    \
        }                                                                                 \
    } while (0)

// Turns a non-zero ngb status into a NeonException carrying ngb_last_error().
#define NEON_NGB_CHECK(expr)                                  \
    do {                                                      \
        int rc_ = (expr);                                     \
        if (rc_ != 0) {                                       \
            ::Neon::NeonException ex_("neon_gb300");          \
            ex_ << #expr << " -> " << rc_ << ": " << ngb_last_error(); \
            throw ex_;                                        \
        }                                                     \
    } while (0)

class Backend {
   public:
    static constexpr int mainStreamIdx = 0;

    Backend() = default;
    Backend(const std::vector<int>& devIds, Runtime runtime)
    {
        if (devIds.size() != 1) {
            NeonException e("Backend");
            e << "this build runs one partition on one GPU; got " << devIds.size() << " device ids";
            NEON_THROW(e);
        }
        if (runtime != Runtime::stream) {
            NeonException e("Backend");
            e << "only Runtime::stream (the GPU) is available; there is no CPU fallback";
            NEON_THROW(e);
        }
        mData = std::make_shared<Data>();
        mData->dev = devIds[0];
        mData->runtime = runtime;
    }

    auto runtime() const -> Runtime { return mData ? mData->runtime : Runtime::none; }
    auto deviceId() const -> int { return mData->dev; }
    auto getDeviceCount() const -> int { return 1; }

    // cudaStream_t of stream index `idx` (created on first use).
    auto stream(int idx = mainStreamIdx) const -> cudaStream_t
    {
        auto it = mData->streams.find(idx);
        if (it != mData->streams.end()) return it->second;
        NEON_CUDA_CHECK(cudaSetDevice(mData->dev));
        cudaStream_t s;
        NEON_CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        mData->streams[idx] = s;
        return s;
    }
    void setDevice() const { NEON_CUDA_CHECK(cudaSetDevice(mData->dev)); }
    void sync(int idx = mainStreamIdx) const { NEON_CUDA_CHECK(cudaStreamSynchronize(stream(idx))); }
    void syncAll() const
    {
        for (auto& kv : mData->streams) NEON_CUDA_CHECK(cudaStreamSynchronize(kv.second));
    }
    bool isInit() const { return mData != nullptr; }

   private:
    struct Data {
        int                         dev = 0;
        Runtime                     runtime = Runtime::stream;
        std::map<int, cudaStream_t> streams;
        ~Data()
        {
            for (auto& kv : streams) cudaStreamDestroy(kv.second);
        }
    };
    std::shared_ptr<Data> mData;
};

}  // namespace Neon
