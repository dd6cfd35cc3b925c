// Stand-in for cub::Sum, which CUDA 13's CUB no longer provides (it names
// cuda::std::plus instead); forced into the reference files that still use it.
#pragma once
#include <cub/cub.cuh>
namespace cub {
struct Sum {
    template <typename A, typename B>
    __host__ __device__ __forceinline__ auto operator()(const A& a, const B& b) const -> decltype(a + b)
    {
        return a + b;
    }
};
}  // namespace cub
