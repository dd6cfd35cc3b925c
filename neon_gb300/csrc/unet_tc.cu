// 3x3x3 BF16 convolution of the learned preconditioner on Blackwell's
// 5th-generation tensor cores (tcgen05), as an implicit GEMM:
//   D[v][co] = sum_{tap t, channel c} x[ngh(v, t)][c] * w[co][t][c]
// M = 128 consecutive voxels (one tile), N = Cout, K = 27 taps x Cin, in
// tcgen05.mma steps of M 128, N Cout, K 16.
//
// Operand staging (TMA, one 5-D box per stage: 8 channels x voxels x all
// Cin / 8 channel groups, so the shared-memory image is already the
// no-swizzle K-major layout: 8-row x 16-byte core matrices, 8-row groups
// 128 B apart (SBO), 8-channel groups one voxel strip apart (LBO)):
//   strip mode (nx % 128 == 0): a stage is one (dy, dz) strip of 130 voxels
//     (x0 - 1 .. x0 + 128) with all channels; the three dx taps are the same
//     image read from rows 0, 1, 2 (start address + 16 B per row), so a tile
//     takes 9 stages and each input voxel is staged 9 times, not 27;
//   tap mode (nx a divisor of 128): a stage is one tap's box of 128 voxels
//     (by = 128 / nx rows of the grid), 27 stages per tile.
// The tensor map's zero fill at the grid faces is the convolution's zero
// padding. The weights of a stage's taps (pre-packed into the B operand
// image) arrive by one bulk copy on the same barrier.
//
// Per CTA (persistent over tiles, 6 warps):
//   warp 0     one thread issues the TMA and bulk copies;
//   warp 1     owns the TMEM accumulators (two buffers of N FP32 columns at
//              column offsets 0 and kCols / 2); one thread issues the MMAs and
//              commits each stage back to the producer and each finished tile
//              to the epilogue;
//   warps 2-5  epilogue: tcgen05.ld of their 32-lane quarter, optional bias /
//              ReLU / accumulation, BF16 or FP32 stores (channels-last rows).
//
// Every wait is bounded: on time-out the kernel raises a device error flag
// (read by ngb_conv3d_tc_check), waits for its own copies and MMAs with the
// same bound, frees its TMEM and returns.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

namespace ngb {
namespace {

constexpr int      kTcM = 128;           // voxels per tile (MMA M)
constexpr int      kTcMaxStages = 8;     // shared-memory pipeline depth (at most)
constexpr int      kTcThreads = 192;     // 6 warps
constexpr int      kStripRows = kTcM + 2;  // voxels x0 - 1 .. x0 + 128
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ int g_tc_error;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase of `parity` to complete; false when this CTA has given up
// (its own limit ran out, or another role's did).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1;
    atomicExch(&g_tc_error, 1);
    return false;
}
// Drain wait used on the way out: bounded, ignores the abort flag.
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity)
{
    for (uint32_t i = 0; i < kWaitLimit; i++)
        if (mbar_try_wait(bar, parity)) return;
    atomicExch(&g_tc_error, 1);
}

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c1, int c2, int c3, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
        "[%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(c1), "r"(c2), "r"(c3), "r"(0), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset
// >> 4 (16-29), stride byte offset >> 4 (32-45), descriptor version 1 (46-47),
// base offset 0, no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) | (uint64_t((sbo >> 4) & 0x3FFFu) << 32) |
           (uint64_t(1) << 46);
}
// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 (bits 17-22), M >> 4 (24-28).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

template <int N>
struct TmemCols {
    static constexpr uint32_t value = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : 256));
};

struct TcParams {
    int                  nx, ny, nz, kc;  // kc = Cin / 16
    int                  strip;           // 1: strip mode, 0: tap mode
    int                  nstages;         // pipeline depth
    uint32_t             a_bytes, b_bytes, stage_bytes;  // per stage (stage_bytes: 128-aligned stride)
    uint32_t             a_lbo;           // bytes between 8-channel groups in the A image (rows * 16)
    int64_t              tiles;
    const __nv_bfloat16* wpk;  // packed weights: per tap Cin / 8 groups of N x 8 BF16
    const float*         bias;
    void*                y;
    int                  ldy, relu, accumulate;
};

template <int N, bool F32OUT>
__global__ void __launch_bounds__(kTcThreads, 1) conv3d_tc_kernel(const __grid_constant__ CUtensorMap xmap, TcParams p)
{
    constexpr uint32_t kCols = TmemCols<N>::value;
    constexpr uint32_t kIdesc = idesc_bf16_f32(kTcM, N);

    extern __shared__ uint8_t smem_raw[];
    uint8_t* stages = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));

    __shared__ uint64_t     full_bar[kTcMaxStages], empty_bar[kTcMaxStages], tfull_bar[2], tempty_bar[2], drain_bar;
    __shared__ uint32_t     tmem_base_sh;
    __shared__ volatile int abort_sh;

    const int      warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ns = uint32_t(p.nstages);
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < ns; s++) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull_bar[a], 1);
            mbar_init(&tempty_bar[a], 4);
        }
        mbar_init(&drain_bar, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)), "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const int      nst = p.strip ? 9 : 27;  // stages per tile
    const int      ntap = p.strip ? 3 : 1;  // taps per stage
    const uint32_t tap_b = uint32_t(N) * uint32_t(p.kc) * 32u;  // B bytes of one tap

    if (warp == 0 && lane == 0) {
        // ------------------------------------------------ TMA producer
        uint32_t k = 0;
        bool     ok = true;
        for (int64_t tile = blockIdx.x; tile < p.tiles && ok; tile += gridDim.x) {
            const int64_t v0 = tile * kTcM;
            const int     x0 = int(v0 % p.nx);
            const int64_t row = v0 / p.nx;
            const int     y0 = int(row % p.ny), z0 = int(row / p.ny);
            for (int i = 0; i < nst; i++, k++) {
                // strip g = 3 (dz + 1) + (dy + 1); tap t = 9 (dz + 1) + 3 (dy + 1) + (dx + 1)
                const int dx = p.strip ? -1 : i % 3 - 1;
                const int dy = (p.strip ? i : i / 3) % 3 - 1, dz = (p.strip ? i / 3 : i / 9) - 1;
                const uint32_t s = k % ns;
                if (!(ok = mbar_wait(&empty_bar[s], ((k / ns) & 1u) ^ 1u, &abort_sh))) break;
                uint8_t* st = stages + size_t(s) * p.stage_bytes;
                mbar_expect_tx(&full_bar[s], p.a_bytes + p.b_bytes);
                tma_load_5d(st, &xmap, x0 + dx, y0 + dy, z0 + dz, &full_bar[s]);
                bulk_load(st + p.stage_bytes - ((p.b_bytes + 127u) & ~127u), reinterpret_cast<const uint8_t*>(p.wpk) + size_t(i) * ntap * tap_b,
                          p.b_bytes, &full_bar[s]);
            }
        }
        // copies still in flight land before the CTA leaves: the latest phase of
        // each stage used is complete once its bytes have arrived
        const uint32_t used = k < ns ? k : ns;
        for (uint32_t j = k - used; j < k; j++) mbar_drain(&full_bar[j % ns], (j / ns) & 1u);
    } else if (warp == 1 && lane == 0) {
        // ------------------------------------------------ MMA issuer
        uint32_t k = 0, j = 0;
        bool     ok = true;
        for (int64_t tile = blockIdx.x; tile < p.tiles && ok; tile += gridDim.x, j++) {
            const uint32_t a = j & 1u, u = (j >> 1) & 1u;
            if (!(ok = mbar_wait(&tempty_bar[a], u ^ 1u, &abort_sh))) break;
            tc_fence_after();
            const uint32_t d = tmem + a * (kCols / 2);  // buffers at power-of-two column offsets
            uint32_t       acc = 0;
            for (int i = 0; i < nst; i++, k++) {
                const uint32_t s = k % ns;
                if (!(ok = mbar_wait(&full_bar[s], (k / ns) & 1u, &abort_sh))) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(stages + size_t(s) * p.stage_bytes);
                const uint32_t sb = sa + p.stage_bytes - ((p.b_bytes + 127u) & ~127u);
                for (int t = 0; t < ntap; t++) {
                    for (int kc = 0; kc < p.kc; kc++) {
                        // A: rows from t (the dx shift of strip mode), channel groups 2kc, 2kc + 1
                        const uint64_t ad = smem_desc(sa + uint32_t(t) * 16u + uint32_t(kc) * 2u * p.a_lbo, p.a_lbo, 128);
                        const uint64_t bd = smem_desc(sb + uint32_t(t) * tap_b + uint32_t(kc) * 2u * N * 16u, N * 16, 128);
                        mma_bf16(d, ad, bd, kIdesc, acc);
                        acc = 1;
                    }
                }
                mma_commit(&empty_bar[s]);
            }
            if (ok) mma_commit(&tfull_bar[a]);
        }
        // every MMA issued here has completed before TMEM is released
        mma_commit(&drain_bar);
        mbar_drain(&drain_bar, 0);
    } else if (warp >= 2) {
        // ------------------------------------------------ epilogue
        const uint32_t q = uint32_t(warp & 3);  // the TMEM lane quarter this warp may read
        uint32_t       j = 0;
        for (int64_t tile = blockIdx.x; tile < p.tiles; tile += gridDim.x, j++) {
            const uint32_t a = j & 1u, u = (j >> 1) & 1u;
            if (!mbar_wait(&tfull_bar[a], u, &abort_sh)) break;
            tc_fence_after();
            float acc[N];
#pragma unroll
            for (int c = 0; c < N; c += 16) tmem_ld16(tmem + ((q * 32u) << 16) + a * (kCols / 2) + c, acc + c);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty_bar[a]);
            const int64_t v = tile * kTcM + q * 32 + lane;
            if (p.bias) {
#pragma unroll
                for (int c = 0; c < N; c++) acc[c] += __ldg(p.bias + c);
            }
            if constexpr (F32OUT) {
                float* yo = static_cast<float*>(p.y) + v * p.ldy;
#pragma unroll
                for (int c = 0; c < N; c += 4) {
                    float4 o = make_float4(acc[c], acc[c + 1], acc[c + 2], acc[c + 3]);
                    if (p.accumulate) {
                        const float4 old = *reinterpret_cast<const float4*>(yo + c);
                        o.x += old.x, o.y += old.y, o.z += old.z, o.w += old.w;
                    }
                    *reinterpret_cast<float4*>(yo + c) = o;
                }
            } else {
                __nv_bfloat16* yo = static_cast<__nv_bfloat16*>(p.y) + v * p.ldy;
#pragma unroll
                for (int c = 0; c < N; c += 8) {
                    uint32_t w4[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        float lo = acc[c + 2 * e], hi = acc[c + 2 * e + 1];
                        if (p.relu) lo = fmaxf(lo, 0.f), hi = fmaxf(hi, 0.f);
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(lo, hi);
                        w4[e] = *reinterpret_cast<const uint32_t*>(&h2);
                    }
                    *reinterpret_cast<uint4*>(yo + c) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

// packed[((t * kc + c16) * 2 + h) * N * 8 + n * 8 + e] = w[n][t][c16 * 16 + h * 8 + e]
__global__ void conv3d_pack_kernel(int cout, int cin, const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ out)
{
    const int64_t total = int64_t(cout) * 27 * cin;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
        const int e = int(i % 8);
        const int n = int((i / 8) % cout);
        const int64_t rest = i / (8 * int64_t(cout));  // (t * kc + c16) * 2 + h
        const int h = int(rest % 2);
        const int64_t tc = rest / 2;
        const int kc = cin / 16;
        const int t = int(tc / kc), c16 = int(tc % kc);
        out[i] = w[(int64_t(n) * 27 + t) * cin + c16 * 16 + h * 8 + e];
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag                    once;
    std::call_once(once, []() {
        void*                           p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <int N, bool F32OUT>
int launch_tc(const CUtensorMap& map, const TcParams& p, cudaStream_t s)
{
    const size_t smem = size_t(p.nstages) * p.stage_bytes + 1024;  // + alignment slack
    NGB_CUDA_TRY(cudaFuncSetAttribute(conv3d_tc_kernel<N, F32OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int dev = 0, sms = 0, per_sm = 0;
    NGB_CUDA_TRY(cudaGetDevice(&dev));
    NGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv3d_tc_kernel<N, F32OUT>, kTcThreads, smem));
    // persistent CTAs: all resident at once (two per SM hold at most 2 x 256 TMEM columns)
    const int64_t grid = std::min<int64_t>(p.tiles, int64_t(sms) * std::max(1, std::min(per_sm, 2)));
    conv3d_tc_kernel<N, F32OUT><<<int(grid), kTcThreads, smem, s>>>(map, p);
    NGB_LAUNCH_CHECK("conv3d_tc_kernel");
    return NGB_OK;
}

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_conv3d_tc_supported(int nx, int ny, int nz, int ldx, int cin, int ldy, int cout)
{
    if (nx < 1 || ny < 1 || nz < 1) return 0;
    if (cin < 16 || cin % 16 != 0 || ldx < cin || ldx % 8 != 0) return 0;
    if (!(cout == 16 || cout == 32 || cout == 48 || cout == 64 || cout == 96) || ldy < cout || ldy % 8 != 0) return 0;
    if (nx % kTcM == 0) return 1;
    return (nx < kTcM && kTcM % nx == 0 && ny % (kTcM / nx) == 0) ? 1 : 0;
}

int ngb_conv3d_pack(int cout, int cin, const void* w, void* packed, void* stream)
{
    NGB_CHECK_ARG(w && packed, "NULL pointer");
    NGB_CHECK_ARG(cout >= 8 && cout % 8 == 0 && cin >= 16 && cin % 16 == 0, "cout must be a multiple of 8, cin of 16");
    const int64_t total = int64_t(cout) * 27 * cin;
    const int     grid = int(std::min<int64_t>((total + 255) / 256, 4096));
    conv3d_pack_kernel<<<grid, 256, 0, as_stream(stream)>>>(cout, cin, static_cast<const __nv_bfloat16*>(w),
                                                            static_cast<__nv_bfloat16*>(packed));
    NGB_LAUNCH_CHECK("conv3d_pack_kernel");
    return NGB_OK;
}

int ngb_conv3d_tc(int nx, int ny, int nz, const void* x, int ldx, int cin, const void* wpacked, const float* bias, void* y, int ldy,
                  int cout, int out_f32, int relu, int accumulate, void* stream)
{
    NGB_CHECK_ARG(x && wpacked && y, "NULL pointer");
    if (!ngb_conv3d_tc_supported(nx, ny, nz, ldx, cin, ldy, cout)) {
        set_error("ngb_conv3d_tc: unsupported shape (nx %d ny %d nz %d ldx %d cin %d ldy %d cout %d)", nx, ny, nz, ldx, cin, ldy,
                  cout);
        return NGB_ERR_UNSUPPORTED;
    }
    NGB_CHECK_ARG(aligned16(x) && aligned16(wpacked) && aligned16(y) && (!bias || aligned16(bias)),
                  "x, packed weights, y and bias must be 16-byte aligned");
    NGB_CHECK_ARG(!accumulate || out_f32, "accumulate needs FP32 output");
    auto encode = tensor_map_encoder();
    if (!encode) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return NGB_ERR_CUDA;
    }
    // 5-D view (8 channels, x, y, z, channel group): one box per stage holds
    // every channel, laid out group-major (the K-major core-matrix image)
    const bool strip = nx % kTcM == 0;
    const int  bx = strip ? kStripRows : nx, by = strip ? 1 : kTcM / nx, rows = bx * by;
    CUtensorMap map;
    cuuint64_t  dims[5] = {8, cuuint64_t(nx), cuuint64_t(ny), cuuint64_t(nz), cuuint64_t(cin / 8)};
    cuuint64_t  strides[4] = {cuuint64_t(ldx) * 2, cuuint64_t(ldx) * 2 * nx, cuuint64_t(ldx) * 2 * nx * ny, 16};
    cuuint32_t  box[5] = {8, cuuint32_t(bx), cuuint32_t(by), 1, cuuint32_t(cin / 8)};
    cuuint32_t  estr[5] = {1, 1, 1, 1, 1};
    const CUresult cr = encode(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x), dims, strides, box, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", int(cr));
        return NGB_ERR_CUDA;
    }
    TcParams p{};
    p.nx = nx, p.ny = ny, p.nz = nz, p.kc = cin / 16;
    p.strip = strip ? 1 : 0;
    p.a_lbo = uint32_t(rows) * 16u;
    p.a_bytes = p.a_lbo * uint32_t(cin / 8);
    p.b_bytes = uint32_t(strip ? 3 : 1) * uint32_t(cout) * uint32_t(cin) * 2u;
    p.stage_bytes = ((p.a_bytes + 127u) & ~127u) + ((p.b_bytes + 127u) & ~127u);
    // depth: as many stages as fit in ~108 KB (two CTAs per SM), 2 to 8
    p.nstages = int(std::min<uint32_t>(kTcMaxStages, std::max<uint32_t>(2u, (108u * 1024u) / p.stage_bytes)));
    p.tiles = int64_t(nx) * ny * nz / kTcM;
    p.wpk = static_cast<const __nv_bfloat16*>(wpacked);
    p.bias = bias, p.y = y, p.ldy = ldy, p.relu = relu, p.accumulate = accumulate;
    if (p.tiles == 0) return NGB_OK;
    cudaStream_t s = as_stream(stream);
#define NGB_TC(NN)                                                   \
    case NN:                                                         \
        return out_f32 ? launch_tc<NN, true>(map, p, s) : launch_tc<NN, false>(map, p, s);
    switch (cout) {
        NGB_TC(16)
        NGB_TC(32)
        NGB_TC(48)
        NGB_TC(64)
        NGB_TC(96)
        default: break;
    }
#undef NGB_TC
    set_error("unsupported cout %d", cout);
    return NGB_ERR_UNSUPPORTED;
}

int ngb_conv3d_tc_check(void* stream)
{
    NGB_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    int flag = 0;
    NGB_CUDA_TRY(cudaMemcpyFromSymbol(&flag, g_tc_error, sizeof(int)));
    if (flag) {
        const int zero = 0;
        NGB_CUDA_TRY(cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)));
        set_error("conv3d_tc_kernel: a pipeline wait ran out (results are invalid)");
        return NGB_ERR_TIMEOUT;
    }
    return NGB_OK;
}

}  // extern "C"
