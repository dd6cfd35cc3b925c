// Grid-independent pieces of libNeonDomain's interface: NghData
// (include/Neon/domain/interface/NghData.h:9-49) and PatternScalar
// (include/Neon/domain/patterns/PatternScalar.h:9-82).
#pragma once
#include <cuda_runtime.h>

#include "Neon/core/core.h"
#include "Neon/set/Backend.h"
#include "neon_gb300.h"

namespace Neon {
namespace domain {

template <typename T>
struct NghData {
    T    value{};
    bool valid = false;
    NghData() = default;
    NEON_CUDA_HOST_DEVICE NghData(const T& v, bool ok) : value(v), valid(ok) {}
    NEON_CUDA_HOST_DEVICE const T& getData() const { return value; }
    NEON_CUDA_HOST_DEVICE bool     isValid() const { return valid; }
    NEON_CUDA_HOST_DEVICE const T& operator()() const { return value; }
    NEON_CUDA_HOST_DEVICE void     set(const T& v, bool ok) { value = v, valid = ok; }
    NEON_CUDA_HOST_DEVICE void     invalidate() { valid = false; }
};

// A device-resident reduction result (FP64 on the device) with a host view.
// operator()() synchronises the backend's main stream and returns the value
// as T (PatternScalar.h:9-82 semantics: the result of the last reduction).
template <typename T>
class PatternScalar {
   public:
    PatternScalar() = default;
    explicit PatternScalar(const Backend& bk)
    {
        mData = std::make_shared<Data>();
        mData->bk = bk;
        bk.setDevice();
        NEON_CUDA_CHECK(cudaMalloc(&mData->dev, sizeof(double)));
        NEON_CUDA_CHECK(cudaMemset(mData->dev, 0, sizeof(double)));
    }
    double* devPtr() const { return mData->dev; }
    double* scratch() const { return mData->scratch; }
    void    ensureScratch(int64_t n)
    {
        const size_t need = ngb_dot_scratch_doubles(n);
        if (need > mData->scratchSize) {
            if (mData->scratch) cudaFree(mData->scratch);
            NEON_CUDA_CHECK(cudaMalloc(&mData->scratch, need * sizeof(double)));
            mData->scratchSize = need;
        }
    }
    T operator()() const
    {
        double v = 0;
        NEON_CUDA_CHECK(cudaMemcpyAsync(&v, mData->dev, sizeof(double), cudaMemcpyDeviceToHost, mData->bk.stream()));
        mData->bk.sync();
        return T(v);
    }
    void set(T v)
    {
        double d = double(v);
        NEON_CUDA_CHECK(cudaMemcpy(mData->dev, &d, sizeof(double), cudaMemcpyHostToDevice));
    }

   private:
    struct Data {
        Backend bk;
        double* dev = nullptr;
        double* scratch = nullptr;
        size_t  scratchSize = 0;
        ~Data()
        {
            if (dev) cudaFree(dev);
            if (scratch) cudaFree(scratch);
        }
    };
    std::shared_ptr<Data> mData;
};

}  // namespace domain
}  // namespace Neon
