// Shared device/host helpers of the neon_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <nvtx3/nvToolsExt.h>

#include "../../include/neon_gb300.h"

namespace ngb {

// ------------------------------------------------------------------ errors
// Every C-ABI entry point returns an ngb status and never throws; the last
// error message is kept per host thread (ngb_last_error()).
void set_error(const char* fmt, ...);
void clear_error();

#define NGB_CHECK_ARG(cond, ...)                 \
    do {                                         \
        if (!(cond)) {                           \
            ::ngb::set_error(__VA_ARGS__);       \
            return NGB_ERR_INVALID;              \
        }                                        \
    } while (0)

#define NGB_CUDA_TRY(expr)                                                                                \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            ::ngb::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return NGB_ERR_CUDA;                                                                          \
        }                                                                                                 \
    } while (0)

// Launch-error check after a <<<>>> launch.
#define NGB_LAUNCH_CHECK(name)                                                                   \
    do {                                                                                         \
        cudaError_t e_ = cudaGetLastError();                                                     \
        if (e_ != cudaSuccess) {                                                                 \
            ::ngb::set_error("launch of %s failed: %s", name, cudaGetErrorString(e_));           \
            return NGB_ERR_CUDA;                                                                 \
        }                                                                                        \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// NVTX range over a host entry point (the counterpart of the reference's
// "Skeleton" / "Graph Iteration" ranges, Skeleton.h:56-65, Graph.cpp:1001-1029):
// visible to Nsight tools, a no-op without one.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ------------------------------------------------------------------ lattices
// D3Q19 in Neon's order (benchmarks/lbm-lid-driven-cavity-flow/src/D3Q19.h:23-44):
// 0..8 go directions, 9 rest, 10..18 the opposites of 0..8.
template <int Q>
struct Lattice;

template <>
struct Lattice<19> {
    static constexpr int Q = 19;
    __host__ __device__ static constexpr int cx(int q)
    {
        constexpr int v[19] = {-1, 0, 0, -1, -1, -1, -1, 0, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0};
        return v[q];
    }
    __host__ __device__ static constexpr int cy(int q)
    {
        constexpr int v[19] = {0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 0, 1, 0, 1, -1, 0, 0, 1, 1};
        return v[q];
    }
    __host__ __device__ static constexpr int cz(int q)
    {
        constexpr int v[19] = {0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 0, 1, 0, 0, 1, -1, 1, -1};
        return v[q];
    }
    __host__ __device__ static constexpr int opp(int q) { return q == 9 ? 9 : (q < 9 ? q + 10 : q - 10); }
    __host__ __device__ static constexpr double w(int q)
    {
        return q == 9 ? 1. / 3. : ((q % 10) < 3 ? 1. / 18. : 1. / 36.);
    }
};

// D3Q27 in the order of apps/lbmMultiRes/lattice.h:14-42: q = 9a + 3b + c with
// digit 0 -> 0, 1 -> -1, 2 -> +1 for (cx, cy, cz); the rest population is q = 0.
template <>
struct Lattice<27> {
    static constexpr int Q = 27;
    __host__ __device__ static constexpr int dig(int d) { return d == 0 ? 0 : (d == 1 ? -1 : 1); }
    __host__ __device__ static constexpr int cx(int q) { return dig(q / 9); }
    __host__ __device__ static constexpr int cy(int q) { return dig((q / 3) % 3); }
    __host__ __device__ static constexpr int cz(int q) { return dig(q % 3); }
    __host__ __device__ static constexpr int flip(int d) { return d == 0 ? 0 : 3 - d; }
    __host__ __device__ static constexpr int opp(int q) { return 9 * flip(q / 9) + 3 * flip((q / 3) % 3) + flip(q % 3); }
    __host__ __device__ static constexpr double w(int q)
    {
        return ((cx(q) != 0) + (cy(q) != 0) + (cz(q) != 0)) == 0   ? 8. / 27.
               : ((cx(q) != 0) + (cy(q) != 0) + (cz(q) != 0)) == 1 ? 2. / 27.
               : ((cx(q) != 0) + (cy(q) != 0) + (cz(q) != 0)) == 2 ? 1. / 54.
                                                                    : 1. / 216.;
    }
};

// ------------------------------------------------------------------ flags
// Packed cell flag: bits 0..26 wall-neighbour mask (bit q set iff the pull
// source x - c_q is not a fluid node), bits 28..31 classification.
__host__ __device__ inline uint32_t flag_mask(uint32_t f) { return f & 0x07ffffffu; }
__host__ __device__ inline int      flag_class(uint32_t f) { return int(f >> 28); }
__host__ __device__ inline uint32_t make_flag(uint32_t mask, int cls) { return (mask & 0x07ffffffu) | (uint32_t(cls) << 28); }

// A node other cells stream from normally (no bounce-back across it).
__host__ __device__ inline bool is_zouhe_class(int c) { return c == NGB_CELL_PRESSURE || c == NGB_CELL_VELOCITY; }
__host__ __device__ inline bool is_fluid_class(int c) { return c == NGB_CELL_BULK || c == NGB_CELL_OUTLET || is_zouhe_class(c); }

// ------------------------------------------------------------------ storage
// The 16-bit "off" forms hold g = f - w_q; FP16 holds it scaled by 2^14
// (NGB_F16OFF_SCALE). log2 of the scale of each stored type:
template <typename S>
struct StoreScale {
    static constexpr int log2 = 0;
};
template <>
struct StoreScale<__half> {
    static constexpr int log2 = 14;
};
// FP16 offsets stored with stochastic rounding (NGB_STORE_F16SR): the same
// 2-byte values as __half, a distinct type so that the kernels pick the store.
struct f16sr_t {
    __half h;
};
template <>
struct StoreScale<f16sr_t> {
    static constexpr int log2 = 14;
};

// Random bits of the F16SR store (the definition in neon_gb300.h, ngb_storage).
__host__ __device__ inline uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// h of the cell pair (i >> 1) in step seed s
__host__ __device__ inline uint32_t dither_hash(int64_t cell, uint32_t seed)
{
    const uint64_t pr = uint64_t(cell) >> 1;
    return mix32(uint32_t(pr) ^ (uint32_t(pr >> 32) * 0x9E3779B1u) ^ (seed * 0x85EBCA77u));
}
__host__ __device__ inline uint32_t dither_word(uint32_t h, int q) { return (h ^ (uint32_t(q) * 0x9E3779B9u)) * 0xC2B2AE35u; }
// 13 bits for the even (lo) / odd (hi) cell of the pair: bits 0-12 and 16-28,
// the bits cvt.rs.f16x2.f32 takes for its low and high result from one word
__host__ __device__ inline uint32_t dither_lo(uint32_t hq) { return hq & 0x1fffu; }
__host__ __device__ inline uint32_t dither_hi(uint32_t hq) { return (hq >> 16) & 0x1fffu; }
static_assert(float(1 << StoreScale<__half>::log2) == NGB_F16OFF_SCALE, "FP16 storage scale");

inline size_t storage_bytes(int storage)
{
    return storage == NGB_STORE_F64 ? 8 : (storage == NGB_STORE_F32 ? 4 : 2);
}

}  // namespace ngb
