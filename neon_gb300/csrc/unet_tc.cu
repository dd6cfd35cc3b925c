// 3x3x3 BF16 convolution of the learned preconditioner on Blackwell's
// 5th-generation tensor cores (tcgen05), as an implicit GEMM:
//   D[v][co] = sum_{tap t, channel c} x[ngh(v, t)][c] * w[co][t][c]
// M = 128 consecutive voxels (one tile), N = Cout, K = 27 taps x Cin, in
// tcgen05.mma steps of M 128, N Cout, K 16 (one 16-channel chunk of one tap).
//
// Operands sit in shared memory in the no-swizzle K-major layout: 8-row x
// 16-byte core matrices, 8-row groups 128 B apart (SBO), the two 8-channel
// groups of a chunk one voxel image apart (LBO). TMA writes that image
// directly: the input is viewed as a 5-D tensor (8 channels, x, y, z,
// channel group) and a box's channel groups are its slowest dimension.
//
// Plane mode (nx % 128 == 0, ny even): a work unit is two tiles on adjacent
// y rows (x0..x0+127 at y0 and y0 + 1). A pipeline stage is one (dz, chunk):
// one TMA box of 4 y rows (y0 - 1 .. y0 + 2) x 130 voxels (x0 - 1 ..
// x0 + 128) x 16 channels, and one bulk copy of the 9 (dy, dx) taps' weight
// slices. Every (tile, dy, dx) is the same image read from row
// (tile + dy + 1, dx + 1) through the descriptor's start address, so a stage
// feeds 18 MMAs and each input row is staged 3 times per two tiles.
// Tap mode (nx a divisor of 128): a work unit is one tile of 128 / nx rows,
// a stage one (tap, chunk) box, one MMA per stage.
// The tensor map's zero fill at the grid faces is the convolution's padding.
//
// Per CTA (persistent over work units, 6 warps):
//   warp 0     one thread issues the TMA and bulk copies;
//   warp 1     owns the TMEM accumulators (two buffers, each holding the
//              unit's tiles side by side); one thread issues the MMAs and
//              commits each stage back to the producer and each finished
//              unit to the epilogue;
//   warps 2-5  epilogue: tcgen05.ld of their 32-lane quarter, optional bias /
//              ReLU / accumulation, BF16 or FP32 stores (channels-last rows).
//
// Every wait is bounded: on time-out the kernel raises a device error flag
// (read by ngb_conv3d_tc_check), waits for its own copies and MMAs with the
// same bound, frees its TMEM and returns.
#include "common.cuh"
#include "tma.cuh"

namespace ngb {
namespace {

constexpr int      kTcM = 128;           // voxels per tile (MMA M)
constexpr int      kTcMaxStages = 8;     // shared-memory pipeline depth (at most)
constexpr int      kTcThreads = 192;     // 6 warps
constexpr int      kStripRows = kTcM + 2;  // plane mode: voxels x0 - 1 .. x0 + 128 of an image row
constexpr int      kZMax = 16;             // z-run mode: output planes per work unit (at most)
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ int g_tc_error;

// Wait for the phase of `parity` to complete; false when this CTA has given up
// (its own limit ran out, or another role's did).
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, volatile int* abort_flag, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1;
    atomicExch(&g_tc_error, 1);
    return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
    return mbar_wait_for(bar, parity, abort_flag, kWaitLimit);
}

// Self-test of the bounded wait: one thread waits, `limit` polls at most, on
// a barrier that nothing arrives on (no copy or MMA is issued), so the wait
// runs out, raises the error flag and returns.
__global__ void tc_wait_selftest_kernel(uint32_t limit, int* gave_up)
{
    __shared__ uint64_t bar;
    __shared__ int      abort_flag;
    mbar_init(&bar, 1);
    abort_flag = 0;
    mbar_init_fence();
    *gave_up = mbar_wait_for(&bar, 0, &abort_flag, limit) ? 0 : 1;
}
// Drain wait used on the way out: bounded, ignores the abort flag.
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity)
{
    for (uint32_t i = 0; i < kWaitLimit; i++)
        if (mbar_try_wait(bar, parity)) return;
    atomicExch(&g_tc_error, 1);
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

// Zeros into 16 TMEM columns of this warp's 32 lanes (z-run accumulators are
// cleared by the epilogue after it has read them).
__device__ __forceinline__ void tmem_zero16(uint32_t taddr)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr),
        "r"(0u)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

template <int N>
struct TmemCols {
    static constexpr uint32_t value = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : 256));
};

struct TcParams {
    int                  nx, ny, nz, kc;  // kc = Cin / 16
    int                  plane;           // 1: plane mode, 0: tap mode
    int                  zrun;            // plane mode: output planes per work unit marched in z (0: one plane)
    int                  ntile;           // tiles per work unit (2 / 1)
    int                  nstages;         // pipeline depth
    uint32_t             tmem_cols;       // allocated TMEM columns (two buffers of ntile * N)
    uint32_t             a_bytes, b_bytes, stage_bytes;  // per stage (stage_bytes: 128-aligned stride)
    uint32_t             a_lbo;           // bytes between the two 8-channel groups of the A image
    int                  a_row;           // plane mode: voxels per image row (130)
    int64_t              units;
    int                  resident;        // 1: all weights stay in shared memory (stages carry A only)
    uint32_t             w_bytes;         // bytes of the packed weights (27 * N * Cin * 2)
    uint32_t             w_region;        // shared bytes reserved for resident weights (1024-aligned)
    const __nv_bfloat16* wpk;  // packed weights (ngb_conv3d_pack)
    const float*         bias;
    void*                y;
    int                  ldy, relu, accumulate;
};

// First voxel and grid coordinates of work unit u.
struct Unit {
    int64_t v0;
    int     x0, y0, z0;
};
__device__ __forceinline__ Unit unit_of(const TcParams& p, int64_t u)
{
    Unit t;
    if (p.plane) {
        const int64_t xt = p.nx / kTcM, yt = p.ny / 2;
        t.x0 = int(u % xt) * kTcM;
        const int64_t r = u / xt;
        t.y0 = int(r % yt) * 2;
        t.z0 = int(r / yt);
        t.v0 = t.x0 + int64_t(p.nx) * (t.y0 + int64_t(p.ny) * t.z0);
    } else {
        t.v0 = u * kTcM;
        t.x0 = int(t.v0 % p.nx);
        const int64_t r = t.v0 / p.nx;
        t.y0 = int(r % p.ny), t.z0 = int(r / p.ny);
    }
    return t;
}

// z-run mode: work unit u covers, on the output planes z0 .. z0 + nzo - 1,
// the two rows y0, y0 + 1 of 128 voxels from x0 (plane mode), or the 128
// consecutive voxels of a plane from (x0, y0) (tap mode).
struct ZUnit {
    int64_t v0;
    int     x0, y0, z0, nzo;
};
__device__ __forceinline__ ZUnit zunit_of(const TcParams& p, int64_t u)
{
    ZUnit t;
    if (p.plane) {
        const int64_t xt = p.nx / kTcM, yt = p.ny / 2;
        t.x0 = int(u % xt) * kTcM;
        const int64_t r = u / xt;
        t.y0 = int(r % yt) * 2;
        t.z0 = int(r / yt) * p.zrun;
    } else {
        const int64_t tpp = int64_t(p.nx) * p.ny / kTcM, vin = (u % tpp) * kTcM;
        t.x0 = int(vin % p.nx);
        t.y0 = int(vin / p.nx);
        t.z0 = int(u / tpp) * p.zrun;
    }
    t.nzo = min(p.zrun, p.nz - t.z0);
    t.v0 = t.x0 + int64_t(p.nx) * (t.y0 + int64_t(p.ny) * t.z0);
    return t;
}

// The 18 MMAs of one plane-mode stage (two output rows x the 9 (dy, dx) taps)
// into the accumulator pair at TMEM column d0. Descriptors are the stage's
// and the weight slices' base descriptors plus compile-time offsets in the
// 16-byte address field: A row (tt + dy) * 130 + dx of the staged image, B
// slice tap (N * 32 bytes each); both stay inside shared memory (< 2^18
// bytes), so the 14-bit field takes the sum without a carry. `acc`: whether
// the first tap adds to the accumulators (the other taps always do).
template <int N>
__device__ __forceinline__ void plane_stage_mmas(uint32_t d0, uint64_t a0, uint64_t b0, uint32_t acc)
{
    constexpr uint32_t kIdesc = idesc_bf16_f32(kTcM, N);
#pragma unroll
    for (int tt = 0; tt < 2; tt++)
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
            constexpr int  kRow = kStripRows;
            const uint64_t ad = a0 + uint64_t((tt + tap / 3) * kRow + tap % 3);
            const uint64_t bd = b0 + uint64_t(tap * (N * 32 / 16));
            mma_bf16(d0 + uint32_t(tt * N), ad, bd, kIdesc, tap > 0 ? 1u : acc);
        }
}

// Epilogue of one output tile: bias, ReLU, FP32 (optionally accumulated) or
// BF16 output of voxel v (this thread's lane of the tile).
template <int N, bool F32OUT>
__device__ __forceinline__ void tc_store(const TcParams& p, int64_t v, float (&acc)[N])
{
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

template <int N, bool F32OUT>
__global__ void __launch_bounds__(kTcThreads, 1) conv3d_tc_kernel(const __grid_constant__ CUtensorMap xmap, TcParams p)
{
    constexpr uint32_t kIdesc = idesc_bf16_f32(kTcM, N);

    extern __shared__ uint8_t smem_raw[];
    uint8_t* wres = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* stages = wres + p.w_region;

    __shared__ uint64_t     full_bar[kTcMaxStages], empty_bar[kTcMaxStages], tfull_bar[kZMax], tempty_bar[kZMax], drain_bar, w_bar;
    __shared__ uint32_t     tmem_base_sh;
    __shared__ volatile int abort_sh;

    const int      warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ns = uint32_t(p.nstages);
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < ns; s++) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        for (int a = 0; a < kZMax; a++) {
            mbar_init(&tfull_bar[a], 1);
            mbar_init(&tempty_bar[a], 4);
        }
        mbar_init(&drain_bar, 1);
        mbar_init(&w_bar, 1);
        abort_sh = 0;
        mbar_init_fence();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(p.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const uint32_t half_cols = p.tmem_cols / 2;           // accumulator buffer 1 starts here
    // z-run mode: tile tt's output plane lo accumulates in TMEM columns
    // tt * zcols + (zrun - 1 - lo) * N; every MMA adds to its columns, which
    // start at zero and are cleared again by the epilogue after each read
    const uint32_t zcols = uint32_t(p.zrun) * N;
    const int      ztiles = p.plane ? 2 : 1;
    if (p.zrun) {
        if (warp >= 2) {
            const uint32_t q = uint32_t(warp & 3);
            for (uint32_t c = 0; c < uint32_t(ztiles) * zcols; c += 16) tmem_zero16(tmem + ((q * 32u) << 16) + c);
            tmem_wait_st();
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    const int      nst = (p.plane ? 3 : 27) * p.kc;       // stages per unit
    const uint32_t slice = uint32_t(N) * 32u;             // B bytes of one (tap, chunk)
    const uint32_t b_off = p.stage_bytes - ((p.b_bytes + 127u) & ~127u);

    if (warp == 0 && lane == 0) {
        // ------------------------------------------------ TMA producer
        if (p.resident && p.zrun) {
            // z-run mode: the three dz slices of each (chunk, tap, K half) side by side, so
            // that one MMA of N = 3 Cout applies an input plane to three output planes:
            // smem[((((c16 * 9 + tap) * 2 + h) * 3 + dz) * N + n) * 8 + e]
            mbar_expect_tx(&w_bar, p.w_bytes);
            const uint32_t blk = uint32_t(N) * 16u;  // bytes of one (dz, c16, tap, h) block
            for (int c16 = 0; c16 < p.kc; c16++)
                for (int tap = 0; tap < 9; tap++)
                    for (int h = 0; h < 2; h++)
                        for (int dz = 0; dz < 3; dz++) {
                            const uint32_t src = uint32_t(((dz * p.kc + c16) * 9 + tap) * 2 + h) * blk;
                            const uint32_t dst = uint32_t(((c16 * 9 + tap) * 2 + h) * 3 + dz) * blk;
                            bulk_load(wres + dst, reinterpret_cast<const uint8_t*>(p.wpk) + src, blk, &w_bar);
                        }
        } else if (p.resident) {  // the whole packed weight image, once
            mbar_expect_tx(&w_bar, p.w_bytes);
            for (uint32_t off = 0; off < p.w_bytes; off += 65536u)  // copies of at most 64 KB
                bulk_load(wres + off, reinterpret_cast<const uint8_t*>(p.wpk) + off, min(65536u, p.w_bytes - off), &w_bar);
        }
        uint32_t k = 0;
        bool     ok = true;
        // z-run mode: every input plane z0 - 1 .. z0 + nzo of the unit once, chunk by chunk
        // (tap mode: once per (dy, dx) tap, the box shifted by it; planes outside the
        // grid read as zeros); the MMA issuer applies each to the three output planes
        // it belongs to
        const int taps = p.plane ? 1 : 9;  // stages per input plane and chunk
        for (int64_t u = blockIdx.x; p.zrun && u < p.units && ok; u += gridDim.x) {
            const ZUnit t = zunit_of(p, u);
            const int   nsu = (t.nzo + 2) * taps * p.kc;
            for (int i = 0; i < nsu; i++, k++) {
                const int      chunk = i % p.kc, tap = (i / p.kc) % taps, pi = i / (p.kc * taps);
                const uint32_t s = k % ns;
                if (!(ok = mbar_wait(&empty_bar[s], ((k / ns) & 1u) ^ 1u, &abort_sh))) break;
                uint8_t* st = stages + size_t(s) * p.stage_bytes;
                mbar_expect_tx(&full_bar[s], p.a_bytes);
                const int dyi = p.plane ? 0 : tap / 3, dxi = p.plane ? 0 : tap % 3;
                tma_load_5d(st, &xmap, 0, t.x0 + dxi - 1, t.y0 + dyi - 1, t.z0 + pi - 1, 2 * chunk, &full_bar[s]);
            }
        }
        for (int64_t u = blockIdx.x; !p.zrun && u < p.units && ok; u += gridDim.x) {
            const Unit t = unit_of(p, u);
            for (int i = 0; i < nst; i++, k++) {
                // plane: i = dz_index * kc + chunk; tap: i = tap * kc + chunk, tap = 9 dz + 3 dy + dx (indices 0..2)
                const int      chunk = i % p.kc, outer = i / p.kc;
                const uint32_t s = k % ns;
                if (!(ok = mbar_wait(&empty_bar[s], ((k / ns) & 1u) ^ 1u, &abort_sh))) break;
                uint8_t* st = stages + size_t(s) * p.stage_bytes;
                mbar_expect_tx(&full_bar[s], p.a_bytes + p.b_bytes);
                size_t boff;
                if (p.plane) {
                    const int dzi = outer;
                    tma_load_5d(st, &xmap, 0, t.x0 - 1, t.y0 - 1, t.z0 + dzi - 1, 2 * chunk, &full_bar[s]);
                    boff = (size_t(dzi) * p.kc + chunk) * 9 * slice;
                } else {
                    const int dzi = outer / 9, dyi = (outer / 3) % 3, dxi = outer % 3;
                    tma_load_5d(st, &xmap, 0, t.x0 + dxi - 1, t.y0 + dyi - 1, t.z0 + dzi - 1, 2 * chunk, &full_bar[s]);
                    boff = ((size_t(dzi) * p.kc + chunk) * 9 + dyi * 3 + dxi) * slice;
                }
                if (!p.resident) bulk_load(st + b_off, reinterpret_cast<const uint8_t*>(p.wpk) + boff, p.b_bytes, &full_bar[s]);
            }
        }
        // copies still in flight land before the CTA leaves: the latest phase of
        // each stage used is complete once its bytes have arrived
        const uint32_t used = k < ns ? k : ns;
        for (uint32_t j = k - used; j < k; j++) mbar_drain(&full_bar[j % ns], (j / ns) & 1u);
        if (p.resident) mbar_drain(&w_bar, 0);
    } else if (warp == 1 && lane == 0) {
        // ------------------------------------------------ MMA issuer
        uint32_t k = 0, j = 0;
        bool     ok = !p.resident || mbar_wait(&w_bar, 0, &abort_sh);
        // z-run mode: input plane pi (z0 - 1 + pi) feeds the output planes lo = pi - j
        // (j = 0, 1, 2: weights of dz index j) that lie in the unit: blocks jlo .. jhi,
        // whose accumulators are adjacent in TMEM, in one MMA of N = (jhi - jlo + 1) Cout
        // per (tile, tap). Output plane lo's columns must have been read and cleared by
        // the epilogue before its first MMA (pi = lo); it is complete after pi = lo + 2.
        uint32_t upar = 0;  // bit lo: parity of the uses of output slot lo so far
        for (int64_t u = blockIdx.x; p.zrun && u < p.units && ok; u += gridDim.x) {
            const ZUnit t = zunit_of(p, u);
            for (int pi = 0; pi < t.nzo + 2 && ok; pi++) {
                const int jlo = max(0, pi - t.nzo + 1), jhi = min(2, pi);
                if (pi < t.nzo) {
                    if (!(ok = mbar_wait(&tempty_bar[pi], ((upar >> pi) & 1u) ^ 1u, &abort_sh))) break;
                    tc_fence_after();
                }
                const uint32_t idesc = idesc_bf16_f32(kTcM, (jhi - jlo + 1) * N);
                const uint32_t dcol = uint32_t(p.zrun - 1 - pi + jlo) * N;
                const int      taps = p.plane ? 1 : 9;
                for (int r = 0; r < taps * p.kc && ok; r++, k++) {
                    const int      chunk = r % p.kc, tap = r / p.kc;
                    const uint32_t s = k % ns;
                    if (!(ok = mbar_wait(&full_bar[s], (k / ns) & 1u, &abort_sh))) break;
                    tc_fence_after();
                    const uint64_t a0 = smem_desc(smem_u32(stages + size_t(s) * p.stage_bytes), p.a_lbo, 128);
                    const uint64_t b0 = smem_desc(smem_u32(wres) + uint32_t(chunk * 9) * (96u * N), 48 * N, 128) +
                                        uint64_t(jlo * N);  // rows of block jlo (16 bytes each, >> 4)
                    if (p.plane) {
#pragma unroll
                        for (int tt = 0; tt < 2; tt++)
#pragma unroll
                            for (int tp = 0; tp < 9; tp++) {
                                const uint64_t ad = a0 + uint64_t((tt + tp / 3) * kStripRows + tp % 3);
                                const uint64_t bd = b0 + uint64_t(tp * 6 * N);  // 96 N bytes per tap, >> 4
                                mma_bf16(tmem + uint32_t(tt) * zcols + dcol, ad, bd, idesc, 1u);
                            }
                    } else {  // tap mode: the stage holds the box of this (dy, dx) tap
                        mma_bf16(tmem + dcol, a0, b0 + uint64_t(tap * 6 * N), idesc, 1u);
                    }
                    mma_commit(&empty_bar[s]);
                    if (r == taps * p.kc - 1 && pi >= 2) {
                        mma_commit(&tfull_bar[pi - 2]);
                        upar ^= 1u << (pi - 2);
                    }
                }
            }
        }
        for (int64_t u = blockIdx.x; !p.zrun && u < p.units && ok; u += gridDim.x, j++) {
            const uint32_t a = j & 1u, ph = (j >> 1) & 1u;
            if (!(ok = mbar_wait(&tempty_bar[a], ph ^ 1u, &abort_sh))) break;
            tc_fence_after();
            const uint32_t d0 = tmem + a * half_cols;
            for (int i = 0; i < nst; i++, k++) {
                const uint32_t s = k % ns;
                if (!(ok = mbar_wait(&full_bar[s], (k / ns) & 1u, &abort_sh))) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(stages + size_t(s) * p.stage_bytes);
                uint32_t       sb = sa + b_off;
                if (p.resident) {  // this stage's weight slices inside the resident image
                    const int chunk = i % p.kc, outer = i / p.kc;
                    const uint32_t slot = p.plane ? uint32_t((outer * p.kc + chunk) * 9)
                                                  : uint32_t(((outer / 9) * p.kc + chunk) * 9 + outer % 9);
                    sb = smem_u32(wres) + slot * slice;
                }
                if (p.plane) {
                    // the first stage of a unit overwrites each tile's accumulator with its first MMA
                    plane_stage_mmas<N>(d0, smem_desc(sa, p.a_lbo, 128), smem_desc(sb, N * 16, 128), i > 0 ? 1u : 0u);
                } else {
                    mma_bf16(d0, smem_desc(sa, p.a_lbo, 128), smem_desc(sb, N * 16, 128), kIdesc, i > 0 ? 1u : 0u);
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
        bool           ok = true;
        uint32_t       upar = 0;  // bit lo: parity of the uses of output slot lo so far
        for (int64_t u = blockIdx.x; p.zrun && u < p.units && ok; u += gridDim.x) {
            const ZUnit t = zunit_of(p, u);
            for (int lo = 0; lo < t.nzo; lo++) {
                if (!(ok = mbar_wait(&tfull_bar[lo], (upar >> lo) & 1u, &abort_sh))) break;
                tc_fence_after();
                for (int tt = 0; tt < ztiles; tt++) {
                    const uint32_t ta = tmem + ((q * 32u) << 16) + uint32_t(tt) * zcols + uint32_t(p.zrun - 1 - lo) * N;
                    float          acc[N];
#pragma unroll
                    for (int c = 0; c < N; c += 16) {
                        tmem_ld16(ta + c, acc + c);
                        tmem_zero16(ta + c);
                    }
                    const int64_t v = t.v0 + int64_t(lo) * p.nx * p.ny + int64_t(tt) * p.nx + q * 32 + lane;
                    tc_store<N, F32OUT>(p, v, acc);
                }
                tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty_bar[lo]);
                upar ^= 1u << lo;
            }
        }
        for (int64_t u = blockIdx.x; !p.zrun && u < p.units; u += gridDim.x, j++) {
            const uint32_t a = j & 1u, ph = (j >> 1) & 1u;
            if (!mbar_wait(&tfull_bar[a], ph, &abort_sh)) break;
            tc_fence_after();
            const Unit t = unit_of(p, u);
            for (int tt = 0; tt < p.ntile; tt++) {
                float acc[N];
#pragma unroll
                for (int c = 0; c < N; c += 16) tmem_ld16(tmem + ((q * 32u) << 16) + a * half_cols + uint32_t(tt) * N + c, acc + c);
                if (tt == p.ntile - 1) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty_bar[a]);
                }
                const int64_t v = t.v0 + int64_t(tt) * p.nx + q * 32 + lane;
                tc_store<N, F32OUT>(p, v, acc);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols) : "memory");
    }
}

// Operand image of weights w[cout][27][cin] (BF16), ordered so that a plane
// stage's 9 taps and a tap stage's slice are contiguous:
// packed[(((((dz * kc + c16) * 3 + dy) * 3 + dx) * 2 + h) * cout + n) * 8 + e] = w[n][9 dz + 3 dy + dx][16 c16 + 8 h + e]
// (dz, dy, dx the tap indices 0..2).
__global__ void conv3d_pack_kernel(int cout, int cin, const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ out)
{
    const int64_t total = int64_t(cout) * 27 * cin;
    const int     kc = cin / 16;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
        const int     e = int(i % 8);
        const int     n = int((i / 8) % cout);
        int64_t       r = i / (8 * int64_t(cout));
        const int     h = int(r % 2);
        r /= 2;
        const int dx = int(r % 3);
        r /= 3;
        const int dy = int(r % 3);
        r /= 3;
        const int c16 = int(r % kc), dz = int(r / kc);
        out[i] = w[(int64_t(n) * 27 + 9 * dz + 3 * dy + dx) * cin + c16 * 16 + h * 8 + e];
    }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <int N, bool F32OUT>
int launch_tc(const CUtensorMap& map, const TcParams& p, cudaStream_t s)
{
    const size_t smem = p.w_region + size_t(p.nstages) * p.stage_bytes + 1024;  // + alignment slack
    NGB_CUDA_TRY(cudaFuncSetAttribute(conv3d_tc_kernel<N, F32OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    // the whole unified L1 / shared array as shared memory: two CTAs per SM where they fit
    NGB_CUDA_TRY(cudaFuncSetAttribute(conv3d_tc_kernel<N, F32OUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      int(cudaSharedmemCarveoutMaxShared)));
    int dev = 0, sms = 0, smem_sm = 0, smem_reserved = 0;
    NGB_CUDA_TRY(cudaGetDevice(&dev));
    NGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NGB_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    NGB_CUDA_TRY(cudaDeviceGetAttribute(&smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    cudaFuncAttributes fa{};
    NGB_CUDA_TRY(cudaFuncGetAttributes(&fa, conv3d_tc_kernel<N, F32OUT>));
    // persistent CTAs, all resident at once: as many per SM as shared memory,
    // registers and TMEM (512 columns) allow, 2 at most
    const int by_smem = smem_sm / int(smem + fa.sharedSizeBytes + size_t(smem_reserved));
    const int by_regs = 65536 / std::max(1, fa.numRegs * kTcThreads);
    const int by_tmem = int(512u / p.tmem_cols);
    const int per_sm = std::max(1, std::min(std::min(by_smem, by_regs), std::min(by_tmem, 2)));
    const int64_t grid = std::min<int64_t>(p.units, int64_t(sms) * per_sm);
    conv3d_tc_kernel<N, F32OUT><<<int(grid), kTcThreads, smem, s>>>(map, p);
    NGB_LAUNCH_CHECK("conv3d_tc_kernel");
    return NGB_OK;
}


// ---------------------------------------------------------------- weight gradient on tcgen05
// dw[co][t][ci] += sum_v dy[v][co] x[v + off(t)][ci] as an implicit GEMM per
// group of taps: M = 128 rows (tap, ci) of the group (128 / Cin taps; rows
// past the group's taps are zero), N = Cout, K = voxels, accumulated in TMEM
// over the CTA's range of voxels in steps of 64 (four MMAs of K 16).
// Operands are K-major (voxels contiguous per row), which the activations'
// channels-last layout is not: four staging warps gather 8 voxels x 8
// channels per thread with 16-byte loads (zero outside the grid), transpose
// the 8 x 8 block in registers (byte permutes) and store it as one 128-byte
// core matrix; a fifth warp owns TMEM and issues the MMAs. The staging warps
// then read their 32-lane quarter of the accumulator and add it to dw
// through a per-CTA partial: each CTA writes its range's sums to its own slice
// of a scratch array, and a second kernel adds the slices to dw in a fixed
// order, so the result does not depend on which CTA finishes first.
constexpr int kWgThreads = 160;
constexpr int kWgK = 64;       // voxels per stage
constexpr int kWgStages = 3;

struct WgParams {
    int                  nx, ny, nz, cin, ldx, lddy;
    int                  taps, groups, splits;
    int64_t              chunks;  // V / kWgK
    uint32_t             a_bytes, stage_bytes, tmem_cols;
    const __nv_bfloat16* x;
    const __nv_bfloat16* dy;
    float*               part;  // [splits][cout][27][cin] partial sums
};

// 8 x 8 BF16 transpose: in[i] holds 8 channels of voxel i; returns, for
// channel e, the 8 voxels' values as one 16-byte row.
__device__ __forceinline__ uint4 wg_row(const uint4 (&in)[8], int e)
{
    const uint32_t sel = (e & 1) ? 0x7632u : 0x5410u;
    uint32_t       w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t* a = reinterpret_cast<const uint32_t*>(&in[2 * k]);
        const uint32_t* b = reinterpret_cast<const uint32_t*>(&in[2 * k + 1]);
        w[k] = __byte_perm(a[e >> 1], b[e >> 1], sel);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ void st_shared_v4(uint8_t* p, uint4 v)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(smem_u32(p)), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w) : "memory");
}

template <int N>
__global__ void __launch_bounds__(kWgThreads, 1) conv3d_wgrad_tc_kernel(WgParams p)
{
    constexpr uint32_t kIdesc = idesc_bf16_f32(kTcM, N);
    extern __shared__ uint8_t smem_raw[];
    uint8_t* stages = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t     full_bar[kWgStages], empty_bar[kWgStages], done_bar, drain_bar;
    __shared__ uint32_t     tmem_base_sh;
    __shared__ volatile int abort_sh;

    const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int     group = blockIdx.x % p.groups, split = blockIdx.x / p.groups;
    const int     t0 = group * p.taps, nt = min(p.taps, 27 - t0), rows = nt * p.cin;
    const int64_t c_begin = int64_t(split) * p.chunks / p.splits, c_end = int64_t(split + 1) * p.chunks / p.splits;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kWgStages; s++) {
            mbar_init(&full_bar[s], 128);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&done_bar, 1);
        mbar_init(&drain_bar, 1);
        abort_sh = 0;
        mbar_init_fence();
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(p.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;

    if (warp < 4) {
        // ------------------------------------------------ staging, then epilogue
        const int  tid = threadIdx.x, rg = tid >> 3, vg = tid & 7;  // row group (8 rows), voxel group (8 voxels)
        const int  m0 = rg * 8;
        const bool arow = m0 < rows;
        const int  tap = t0 + (arow ? m0 / p.cin : 0), ci0 = arow ? m0 % p.cin : 0;
        const int  dxi = tap % 3 - 1, dyi = (tap / 3) % 3 - 1, dzi = tap / 9 - 1;
        const bool brow = rg < N / 8;
        uint32_t   k = 0;
        bool       ok = true;
        for (int64_t c = c_begin; c < c_end; c++, k++) {
            const uint32_t s = k % kWgStages;
            if (!(ok = mbar_wait(&empty_bar[s], ((k / kWgStages) & 1u) ^ 1u, &abort_sh))) break;
            uint8_t*      st = stages + size_t(s) * p.stage_bytes;
            const int64_t v0 = c * kWgK + vg * 8;  // x of v0 is a multiple of 8 (nx % 8 == 0)
            const int     x0 = int(v0 % p.nx);
            const int64_t yz = v0 / p.nx;
            const int     y = int(yz % p.ny), z = int(yz / p.ny);
            uint4         in[8];
            {
                const int  yy = y + dyi, zz = z + dzi;
                const bool yzok = arow && yy >= 0 && yy < p.ny && zz >= 0 && zz < p.nz;
                const int64_t rowv = (int64_t(zz) * p.ny + yy) * p.nx;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int xx = x0 + i + dxi;
                    in[i] = (yzok && xx >= 0 && xx < p.nx)
                                ? __ldg(reinterpret_cast<const uint4*>(p.x + (rowv + xx) * p.ldx + ci0))
                                : make_uint4(0u, 0u, 0u, 0u);
                }
            }
            uint8_t* dA = st + (vg >> 1) * 4096 + (vg & 1) * 2048 + rg * 128;
#pragma unroll
            for (int e = 0; e < 8; e++) st_shared_v4(dA + e * 16, wg_row(in, e));
            if (brow) {
#pragma unroll
                for (int i = 0; i < 8; i++) in[i] = __ldg(reinterpret_cast<const uint4*>(p.dy + (v0 + i) * p.lddy + rg * 8));
                uint8_t* dB = st + p.a_bytes + (vg >> 1) * (N * 32) + (vg & 1) * (N * 16) + rg * 128;
#pragma unroll
                for (int e = 0; e < 8; e++) st_shared_v4(dB + e * 16, wg_row(in, e));
            }
            // generic-proxy stores made visible to the tensor core (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&full_bar[s]);
        }
        if (ok && c_end > c_begin && mbar_wait(&done_bar, 0, &abort_sh)) {
            tc_fence_after();
            float acc[N];
#pragma unroll
            for (int c = 0; c < N; c += 16) tmem_ld16(tmem + ((uint32_t(warp) * 32u) << 16) + uint32_t(c), acc + c);
            const int m = warp * 32 + lane;
            if (m < rows) {
                const int t = t0 + m / p.cin, ci = m % p.cin;
                float*    part = p.part + int64_t(split) * N * 27 * p.cin;
#pragma unroll
                for (int co = 0; co < N; co++) part[(int64_t(co) * 27 + t) * p.cin + ci] = acc[co];
            }
        }
    } else if (lane == 0) {
        // ------------------------------------------------ MMA issuer (warp 4)
        uint32_t k = 0;
        bool     ok = true;
        for (int64_t c = c_begin; c < c_end; c++, k++) {
            const uint32_t s = k % kWgStages;
            if (!(ok = mbar_wait(&full_bar[s], (k / kWgStages) & 1u, &abort_sh))) break;
            tc_fence_after();
            const uint32_t sa = smem_u32(stages + size_t(s) * p.stage_bytes), sb = sa + p.a_bytes;
#pragma unroll
            for (int mm = 0; mm < kWgK / 16; mm++)
                mma_bf16(tmem, smem_desc(sa + uint32_t(mm) * 4096u, 2048, 128), smem_desc(sb + uint32_t(mm) * (N * 32), N * 16, 128),
                         kIdesc, (k > 0 || mm > 0) ? 1u : 0u);
            mma_commit(&empty_bar[s]);
        }
        if (ok) mma_commit(&done_bar);
        // every MMA issued here has completed before TMEM is released
        mma_commit(&drain_bar);
        mbar_drain(&drain_bar, 0);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols) : "memory");
    }
}

// dw[i] += sum over s of part[s][i], s ascending.
__global__ void wgrad_reduce_kernel(int64_t n, int splits, const float* __restrict__ part, float* __restrict__ dw)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        float acc = 0.f;
        for (int sp = 0; sp < splits; sp++) acc += part[int64_t(sp) * n + i];
        dw[i] += acc;
    }
}

// Scratch of the partial sums, per device, grown on demand and kept.
struct WgScratch {
    std::mutex m;
    float*     ptr[64] = {};
    size_t     bytes[64] = {};
};
WgScratch g_wg_scratch;

template <int N>
int launch_wgrad(WgParams p, float* dw, cudaStream_t s)
{
    const int64_t n = int64_t(N) * 27 * p.cin;
    const size_t  need = size_t(p.splits) * size_t(n) * sizeof(float);
    int           dev = 0;
    NGB_CUDA_TRY(cudaGetDevice(&dev));
    NGB_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d", dev);
    {
        std::lock_guard<std::mutex> lock(g_wg_scratch.m);
        if (g_wg_scratch.bytes[dev] < need) {
            if (g_wg_scratch.ptr[dev]) {
                NGB_CUDA_TRY(cudaStreamSynchronize(s));
                cudaFree(g_wg_scratch.ptr[dev]);
                g_wg_scratch.ptr[dev] = nullptr;
                g_wg_scratch.bytes[dev] = 0;
            }
            NGB_CUDA_TRY(cudaMalloc(&g_wg_scratch.ptr[dev], need));
            g_wg_scratch.bytes[dev] = need;
        }
        p.part = g_wg_scratch.ptr[dev];
    }
    const size_t smem = size_t(kWgStages) * p.stage_bytes + 1024;
    NGB_CUDA_TRY(cudaFuncSetAttribute(conv3d_wgrad_tc_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    conv3d_wgrad_tc_kernel<N><<<p.groups * p.splits, kWgThreads, smem, s>>>(p);
    NGB_LAUNCH_CHECK("conv3d_wgrad_tc_kernel");
    wgrad_reduce_kernel<<<int(std::min<int64_t>((n + 255) / 256, 1024)), 256, 0, s>>>(n, p.splits, p.part, dw);
    NGB_LAUNCH_CHECK("wgrad_reduce_kernel");
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
    // 5-D view (8 channels, x, y, z, channel group); a box holds one
    // 16-channel chunk (two groups), laid out group-major
    const bool plane = nx % kTcM == 0 && ny % 2 == 0;
    const int  bx = plane ? kStripRows : (nx >= kTcM ? kTcM : nx);
    const int  by = plane ? 4 : kTcM / bx;
    CUtensorMap map;
    cuuint64_t  dims[5] = {8, cuuint64_t(nx), cuuint64_t(ny), cuuint64_t(nz), cuuint64_t(cin / 8)};
    cuuint64_t  strides[4] = {cuuint64_t(ldx) * 2, cuuint64_t(ldx) * 2 * nx, cuuint64_t(ldx) * 2 * nx * ny, 16};
    cuuint32_t  box[5] = {8, cuuint32_t(bx), cuuint32_t(by), 1, 2};
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
    p.plane = plane ? 1 : 0;
    p.ntile = plane ? 2 : 1;
    p.a_row = bx;
    p.a_lbo = uint32_t(bx * by) * 16u;
    p.a_bytes = p.a_lbo * 2u;
    p.w_bytes = uint32_t(27 * cout * cin * 2);
    // most layers: weights loaded once per CTA (two CTAs per SM); a plane-mode layer
    // with Cout 16 / 32 keeps up to 168 KB of weights resident at one CTA per SM,
    // which lets it run in z-run mode
    const bool big_resident = plane && (cout == 16 || cout == 32) && p.w_bytes <= 168u * 1024u;
    p.resident = (p.w_bytes <= 56u * 1024u || big_resident) ? 1 : 0;
    p.w_region = p.resident ? (p.w_bytes + 1023u) & ~1023u : 0u;
    p.b_bytes = p.resident ? 0u : uint32_t(plane ? 9 : 1) * uint32_t(cout) * 32u;
    p.stage_bytes = ((p.a_bytes + 127u) & ~127u) + ((p.b_bytes + 127u) & ~127u);
    // z-run mode (resident weights, Cout 16 / 32): a unit marches over zr output
    // planes and stages each input plane once instead of three times; its
    // accumulators (zr planes x the unit's tiles x Cout columns) fill at most
    // 256 TMEM columns, so two CTAs per SM keep fitting
    const bool zrun = p.resident && (cout == 16 || cout == 32);
    const int  ztiles = plane ? 2 : 1;
    int        zr = 0;
    if (zrun) {
        int dev = 0, sms = 152;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
        const int64_t cols2d = plane ? int64_t(nx / kTcM) * (ny / 2) : int64_t(nx) * ny / kTcM;
        zr = std::min(kZMax, 256 / (ztiles * cout));  // plane mode 8 / 4 planes at Cout 16 / 32, tap mode 16 / 8
        // shorter runs while the units would not give every CTA (two per SM) four of them
        while (zr > 2 && cols2d * ((nz + zr - 1) / zr) < int64_t(8) * sms) zr /= 2;
    }
    p.zrun = zr;
    uint32_t cols = 32;
    while (cols < uint32_t(zr ? ztiles * zr * cout : 2 * p.ntile * cout)) cols *= 2;
    p.tmem_cols = cols;
    // depth: as many stages as fit in ~108 KB (two CTAs per SM) or ~200 KB (one), 2 to 8
    const uint32_t budget = (cols <= 256 && p.w_region <= 56u * 1024u ? 108u * 1024u : 200u * 1024u) - p.w_region;
    p.nstages = int(std::min<uint32_t>(kTcMaxStages, std::max<uint32_t>(2u, budget / p.stage_bytes)));
    p.units = plane ? int64_t(nx / kTcM) * (ny / 2) * (zr ? (nz + zr - 1) / zr : nz)
                    : (zr ? int64_t(nx) * ny / kTcM * ((nz + zr - 1) / zr) : int64_t(nx) * ny * nz / kTcM);
    p.wpk = static_cast<const __nv_bfloat16*>(wpacked);
    p.bias = bias, p.y = y, p.ldy = ldy, p.relu = relu, p.accumulate = accumulate;
    if (p.units == 0) return NGB_OK;
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

int ngb_conv3d_bwd_weight_tc_supported(int32_t nx, int32_t ny, int32_t nz, int32_t ldx, int32_t cin, int32_t lddy, int32_t cout)
{
    const int64_t V = int64_t(nx) * ny * nz;
    return nx > 0 && ny > 0 && nz > 0 && nx % 8 == 0 && V % kWgK == 0 && cin % 8 == 0 && cin <= 128 && ldx % 8 == 0 &&
           ldx >= cin && lddy % 8 == 0 && lddy >= cout && (cout == 16 || cout == 32 || cout == 64);
}

int ngb_conv3d_bwd_weight_tc(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* dy,
                             int32_t lddy, int32_t cout, float* dw, void* stream)
{
    NGB_CHECK_ARG(x && dy && dw, "NULL argument");
    if (!ngb_conv3d_bwd_weight_tc_supported(nx, ny, nz, ldx, cin, lddy, cout)) {
        set_error("ngb_conv3d_bwd_weight_tc: unsupported shape (nx %d ny %d nz %d ldx %d cin %d lddy %d cout %d)", nx, ny, nz, ldx,
                  cin, lddy, cout);
        return NGB_ERR_UNSUPPORTED;
    }
    NGB_CHECK_ARG(aligned16(x) && aligned16(dy), "x and dy must be 16-byte aligned");
    int dev = 0, sms = 0;
    NGB_CUDA_TRY(cudaGetDevice(&dev));
    NGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    WgParams p{};
    p.nx = nx, p.ny = ny, p.nz = nz, p.cin = cin, p.ldx = ldx, p.lddy = lddy;
    p.taps = std::min(27, kTcM / cin);
    p.groups = (27 + p.taps - 1) / p.taps;
    p.chunks = int64_t(nx) * ny * nz / kWgK;
    // voxel ranges per tap group: about two CTAs per SM in all, at least 8 stages each
    p.splits = int(std::max<int64_t>(1, std::min<int64_t>(p.chunks / 8, (2 * int64_t(sms) + p.groups - 1) / p.groups)));
    p.a_bytes = 4u * 4096u;
    p.stage_bytes = (p.a_bytes + 4u * uint32_t(cout) * 32u + 1023u) & ~1023u;
    p.tmem_cols = cout <= 32 ? 32u : 64u;
    p.x = static_cast<const __nv_bfloat16*>(x);
    p.dy = static_cast<const __nv_bfloat16*>(dy);
    cudaStream_t s = as_stream(stream);
    switch (cout) {
        case 16: return launch_wgrad<16>(p, dw, s);
        case 32: return launch_wgrad<32>(p, dw, s);
        default: return launch_wgrad<64>(p, dw, s);
    }
}

int ngb_conv3d_tc_wait_selftest(int32_t limit, void* stream)
{
    NGB_CHECK_ARG(limit >= 1 && limit <= (1 << 20), "limit %d out of [1, 2^20]", limit);
    int* gave_up = nullptr;
    NGB_CUDA_TRY(cudaMalloc(&gave_up, sizeof(int)));
    cudaStream_t s = as_stream(stream);
    tc_wait_selftest_kernel<<<1, 1, 0, s>>>(uint32_t(limit), gave_up);
    cudaError_t e = cudaGetLastError();
    int         host = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, gave_up, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(gave_up);
    if (e != cudaSuccess) {
        set_error("wait self-test: %s", cudaGetErrorString(e));
        return NGB_ERR_CUDA;
    }
    if (!host) {
        set_error("wait self-test: the wait completed on a barrier nothing arrived on");
        return NGB_ERR_CUDA;
    }
    return NGB_OK;
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
