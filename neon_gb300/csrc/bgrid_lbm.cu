// bGrid LBM step, momentum-exchange drag and the flow-over-sphere geometry.
// Compiled with --fmad=false (the FP32 step shares the explicit IEEE
// sequence of the dense kernel; FP64 keeps the reference operation order).
#include "bgrid.cuh"
#include "lbm_shifted.cuh"
#include <mutex>
#include <random>
#include <vector>

namespace ngb {
namespace {

template <typename C>
struct BParams {
    C               omega;
    C               wall[2][27];
    const uint32_t* mask;
    const uint32_t* conn;
};

template <typename S>
__device__ __forceinline__ double as_f(S v, double w);
template <>
__device__ __forceinline__ double as_f<double>(double v, double) { return v; }
template <>
__device__ __forceinline__ double as_f<float>(float v, double) { return v; }
template <>
__device__ __forceinline__ double as_f<__half>(__half v, double w)
{
    return double(__half2float(v) * (1.0f / NGB_F16OFF_SCALE)) + double(float(w));
}
template <>
__device__ __forceinline__ double as_f<__nv_bfloat16>(__nv_bfloat16 v, double w)
{
    return double(__bfloat162float(v)) + double(float(w));
}

// Pull source of direction q for voxel (i,j,k): the voxel (i,j,k) - c_q, in
// this block or one of its 26 neighbours (bPartition::helpGetNghIdx,
// bPartition_imp.h:135-309). Every thread takes the same arithmetic path: the
// block offset per axis is -1 / 0 / +1 from the shifted coordinate, the block
// comes from the connectivity row in shared memory (entry 13 is the block
// itself), so a warp that mixes block-edge and inner voxels does not diverge.
template <int Q>
__device__ __forceinline__ uint32_t bgrid_pull_src(const uint32_t* sconn, int i, int j, int k, int q, int& nv)
{
    using L = Lattice<Q>;
    const int cx = L::cx(q), cy = L::cy(q), cz = L::cz(q);
    const int ii = i - cx, jj = j - cy, kk = k - cz;
    const int fx = cx > 0 ? (ii >> 31) : (cx < 0 ? (ii >> 3) : 0);
    const int fy = cy > 0 ? (jj >> 31) : (cy < 0 ? (jj >> 3) : 0);
    const int fz = cz > 0 ? (kk >> 31) : (cz < 0 ? (kk >> 3) : 0);
    nv = (ii & 7) | ((jj & 7) << 3) | ((kk & 7) << 6);
    return sconn[13 + fx + 3 * fy + 9 * fz];
}

// Moving-wall bits of the masked directions (source voxel active and of class
// moving wall). The mask word and the flag of the source are loaded together.
template <int Q>
__device__ __forceinline__ uint32_t bgrid_lidbits(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ mask,
                                                  const uint32_t* sconn, int i, int j, int k, uint32_t m)
{
    uint32_t lid = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (!(m & (1u << q))) continue;
        int            nv;
        const uint32_t nb = bgrid_pull_src<Q>(sconn, i, j, k, q, nv);
        if (nb == NGB_BGRID_NO_BLOCK) continue;
        const uint32_t word = __ldg(mask + size_t(nb) * 16 + (nv >> 5));
        const uint32_t fl = __ldg(flags + size_t(nb) * kBlockVoxels + nv);
        if (((word >> (nv & 31)) & 1u) && flag_class(fl) == NGB_CELL_MOVINGWALL) lid |= 1u << q;
    }
    return lid;
}

// Source pointer of direction q for this voxel: the pulled neighbour
// population, or the voxel's own opposite population when q is masked (the
// half-way bounce-back rule). A source outside every block is taken as a wall,
// so no flag word can make the kernel read outside the field.
template <int Q, typename S>
__device__ __forceinline__ const S* bgrid_src(const S* __restrict__ fin, const uint32_t* sconn, size_t bq, int v, int i, int j,
                                              int k, int q, uint32_t m, bool& masked)
{
    using L = Lattice<Q>;
    if (L::cx(q) == 0 && L::cy(q) == 0 && L::cz(q) == 0) {
        masked = false;
        return fin + (bq + q) * kBlockVoxels + v;
    }
    int            nv;
    const uint32_t nb = bgrid_pull_src<Q>(sconn, i, j, k, q, nv);
    masked = ((m >> q) & 1u) || nb == NGB_BGRID_NO_BLOCK;
    return masked ? fin + (bq + L::opp(q)) * kBlockVoxels + v : fin + (size_t(nb) * Q + q) * kBlockVoxels + nv;
}

// Outlet voxel (zero-gradient outflow): copy the populations of the x-1
// neighbour when it is a valid voxel.
template <int Q, typename S>
__device__ __forceinline__ void bgrid_outlet(const S* __restrict__ fin, S* __restrict__ fout, const uint32_t* mask,
                                             const uint32_t* conn, uint32_t b, int v, int i, int j, int k)
{
    uint32_t     nb;
    int          nv;
    const size_t bq = size_t(b) * Q;
    if (bgrid_valid_ngh(mask, conn, b, i, j, k, -1, 0, 0, nb, nv)) {
#pragma unroll
        for (int q = 0; q < Q; q++) fout[(bq + q) * kBlockVoxels + v] = fin[(size_t(nb) * Q + q) * kBlockVoxels + nv];
    }
}

// One thread per voxel, each pull source resolved per direction (FP64 with
// the reference's operation order, or the FP32 shifted form).
template <int Q, typename S, bool F64>
__global__ void __launch_bounds__(kBlockVoxels, F64 ? 1 : (Q == 19 ? 4 : 3)) bgrid_lbm_kernel(const S* __restrict__ fin, S* __restrict__ fout,
                                                                 const uint32_t* __restrict__ flags,
                                                                 BParams<typename std::conditional<F64, double, float>::type> p)
{
    using L = Lattice<Q>;
    const uint32_t      b = blockIdx.x;
    const int           v = threadIdx.x, i = v & 7, j = (v >> 3) & 7, k = v >> 6;
    __shared__ uint32_t sconn[27];  // this block's neighbour blocks
    if (v < 27) sconn[v] = __ldg(p.conn + size_t(b) * 27 + v);
    const uint32_t f = __ldg(flags + size_t(b) * kBlockVoxels + v);
    __syncthreads();
    const int    cls = flag_class(f);
    const size_t bq = size_t(b) * Q;
    if (cls == NGB_CELL_OUTLET) {
        bgrid_outlet<Q, S>(fin, fout, p.mask, p.conn, b, v, i, j, k);
        return;
    }
    if (cls != NGB_CELL_BULK) return;
    const uint32_t m = flag_mask(f);
    const uint32_t lid = m ? bgrid_lidbits<Q>(flags, p.mask, sconn, i, j, k, m) : 0u;

    if constexpr (F64) {
        S pop[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) {
            bool      masked;
            const S*  src = bgrid_src<Q, S>(fin, sconn, bq, v, i, j, k, q, m, masked);
            const int o = L::opp(q);
            pop[q] = __ldg(src);
            if (masked) pop[q] = pop[q] + S((lid >> q) & 1u ? p.wall[1][o] : p.wall[0][o]);
        }
        S out[Q];
        bgk_f64_ref<Q, S>(pop, p.omega, out);
#pragma unroll
        for (int q = 0; q < Q; q++) fout[(bq + q) * kBlockVoxels + v] = out[q];
    } else {
        float g[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) {
            bool      masked;
            const S*  src = bgrid_src<Q, S>(fin, sconn, bq, v, i, j, k, q, m, masked);
            const int o = L::opp(q);
            // w(opp q) == w(q), so one conversion serves both cases
            g[q] = PairIO<S>::to_g1(__ldg(src), float(L::w(q)));
            if (masked) g[q] = g[q] + ((lid >> q) & 1u ? p.wall[1][o] : p.wall[0][o]);
        }
        bgk_shifted<Q, float, StoreScale<S>::log2>(g, p.omega);
#pragma unroll
        for (int q = 0; q < Q; q++) PairIO<S>::store1(fout + (bq + q) * kBlockVoxels + v, g[q], float(L::w(q)));
    }
}

// ---------------------------------------------------------------- staged step (16-bit D3Q19)
// Each moving direction q gets a cube in shared memory (x pitch 10, 9 rows,
// 9 planes) holding every value the block's voxels pull along q: voxel
// (i,j,k)'s own population q sits at (i + [cx != 0], j + [cy > 0],
// k + [cz > 0]), so the source (i,j,k) - c_q of every voxel falls inside the
// cube, and for an even i on an even x: a voxel pair (i, i+1) pulls each
// direction with one 32-bit shared load. The cube cells that are not own
// positions (the halo: 64 per face direction, 120 per edge direction) come
// from the neighbour blocks through a compile-time table (cube index,
// neighbour slot, source element) walked by the block's threads. One thread
// per x-pair: the collision runs on FP32x2 pairs (per lane the scalar
// sequence, so the results equal the per-voxel kernel's bit for bit) and each
// direction is stored as one 32-bit word per pair. All global loads of a
// thread (own pairs, halo values) are issued before its first shared store.
constexpr int kPX = 10, kPY = 9, kCubeP = kPX * kPY * 9;
constexpr int kStagedThreads = kBlockVoxels / 2;

template <int Q>
__host__ __device__ constexpr bool is_rest(int q)
{
    return Lattice<Q>::cx(q) == 0 && Lattice<Q>::cy(q) == 0 && Lattice<Q>::cz(q) == 0;
}
template <int Q>
__host__ __device__ constexpr int rest_dir()
{
    int r = 0;
    for (int q = 0; q < Q; q++)
        if (is_rest<Q>(q)) r = q;
    return r;
}
// Index of a moving direction among the moving directions (q order).
template <int Q>
__host__ __device__ constexpr int moving_index(int q)
{
    int n = 0;
    for (int p = 0; p < q; p++) n += is_rest<Q>(p) ? 0 : 1;
    return n;
}
__host__ __device__ constexpr int cube_voxel(int i, int j, int k) { return i + kPX * j + kPX * kPY * k; }
// Cube offset of a voxel's own population along q, and of its pull source.
template <int Q>
__host__ __device__ constexpr int cube_own(int q)
{
    return moving_index<Q>(q) * kCubeP + cube_voxel(Lattice<Q>::cx(q) != 0, Lattice<Q>::cy(q) > 0, Lattice<Q>::cz(q) > 0);
}
template <int Q>
__host__ __device__ constexpr int cube_src(int q)
{
    return cube_own<Q>(q) - cube_voxel(Lattice<Q>::cx(q), Lattice<Q>::cy(q), Lattice<Q>::cz(q));
}
template <int Q>
constexpr int halo_count()
{
    int n = 0;
    for (int q = 0; q < Q; q++) {
        if (is_rest<Q>(q)) continue;
        const int in = (Lattice<Q>::cx(q) ? 7 : 8) * (Lattice<Q>::cy(q) ? 7 : 8) * (Lattice<Q>::cz(q) ? 7 : 8);
        n += kBlockVoxels - in;
    }
    return n;
}

// Halo cells: dst = cube index | neighbour slot << 16 (slot (fx+1) + 3(fy+1) +
// 9(fz+1) of the connectivity row), src = q * 512 + voxel in that block.
template <int Q>
struct HaloTable {
    static constexpr int n = halo_count<Q>();
    uint2                e[n];  // {dst, src}: one 8-byte load per entry
};

template <int Q>
constexpr HaloTable<Q> make_halo_table()
{
    HaloTable<Q> t{};
    int          n = 0;
    for (int q = 0; q < Q; q++) {
        if (is_rest<Q>(q)) continue;
        const int cx = Lattice<Q>::cx(q), cy = Lattice<Q>::cy(q), cz = Lattice<Q>::cz(q);
        for (int k = 0; k < 8; k++)
            for (int j = 0; j < 8; j++)
                for (int i = 0; i < 8; i++) {
                    const int si = i - cx, sj = j - cy, sk = k - cz;
                    const int fx = si < 0 ? -1 : (si > 7 ? 1 : 0), fy = sj < 0 ? -1 : (sj > 7 ? 1 : 0),
                              fz = sk < 0 ? -1 : (sk > 7 ? 1 : 0);
                    if (fx == 0 && fy == 0 && fz == 0) continue;
                    const int cube = cube_src<Q>(q) + cube_voxel(i, j, k);
                    const int slot = (fx + 1) + 3 * (fy + 1) + 9 * (fz + 1);
                    const int nv = (si - 8 * fx) + 8 * (sj - 8 * fy) + 64 * (sk - 8 * fz);
                    t.e[n] = uint2{uint32_t(cube) | (uint32_t(slot) << 16), uint32_t(q * kBlockVoxels + nv)};
                    n++;
                }
    }
    return t;
}

__device__ const HaloTable<19> g_halo19 = make_halo_table<19>();

__device__ __forceinline__ __half        lo_of(__half2 w) { return __low2half(w); }
__device__ __forceinline__ __half        hi_of(__half2 w) { return __high2half(w); }
__device__ __forceinline__ __nv_bfloat16 lo_of(__nv_bfloat162 w) { return __low2bfloat16(w); }
__device__ __forceinline__ __nv_bfloat16 hi_of(__nv_bfloat162 w) { return __high2bfloat16(w); }

template <typename S>
constexpr size_t staged_smem()
{
    return size_t(18) * kCubeP * sizeof(S);
}

template <typename S>
__global__ void __launch_bounds__(kStagedThreads, 4)
    bgrid_lbm_staged_kernel(const S* __restrict__ fin, S* __restrict__ fout, const uint32_t* __restrict__ flags, BParams<float> p)
{
    constexpr int Q = 19;
    using L = Lattice<Q>;
    using W = typename PairIO<S>::Word;
    constexpr int kHalo = HaloTable<Q>::n, kPer = (kHalo + kStagedThreads - 1) / kStagedThreads;
    extern __shared__ __align__(16) uint8_t smem_raw[];
    S*                  st = reinterpret_cast<S*>(smem_raw);
    __shared__ uint32_t sconn[27];
    __shared__ uint32_t smissing;  // bit s set: neighbour slot s has no block

    const uint32_t b = blockIdx.x;
    const int      t = threadIdx.x, i = 2 * (t & 3), j = (t >> 2) & 7, k = t >> 5, v = i + 8 * j + 64 * k;
    if (t < 32) {
        const uint32_t nb = t < 27 ? __ldg(p.conn + size_t(b) * 27 + t) : 0u;
        if (t < 27) sconn[t] = nb;
        const uint32_t miss = __ballot_sync(0xffffffffu, t < 27 && nb == NGB_BGRID_NO_BLOCK);
        if (t == 0) smissing = miss;
    }
    const uint2 fl = __ldg(reinterpret_cast<const uint2*>(flags + size_t(b) * kBlockVoxels + v));
    // own populations of the pair, and this thread's halo table entries
    const S* own = fin + size_t(b) * Q * kBlockVoxels + v;
    W        ov[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) ov[q] = __ldg(reinterpret_cast<const W*>(own + q * kBlockVoxels));
    uint32_t hd[kPer], hs[kPer];
#pragma unroll
    for (int r = 0; r < kPer; r++) {
        const int it = t + r * kStagedThreads;
        const uint2 te = it < kHalo ? __ldg(&g_halo19.e[it]) : uint2{0xffffffffu, 0u};
        hd[r] = te.x;
        hs[r] = te.y;
    }
    // halo values (a missing neighbour block leaves its cells unset: every
    // voxel pulling from one treats the direction as a wall); the neighbour
    // comes from the block's connectivity row directly (the CTA's threads
    // share it through L1), so no barrier waits for the row in shared memory
    S hv[kPer];
#pragma unroll
    for (int r = 0; r < kPer; r++) {
        const uint32_t nb = hd[r] != 0xffffffffu ? __ldg(p.conn + size_t(b) * 27 + (hd[r] >> 16)) : NGB_BGRID_NO_BLOCK;
        if (nb == NGB_BGRID_NO_BLOCK) hd[r] = 0xffffffffu;
        hv[r] = nb != NGB_BGRID_NO_BLOCK ? __ldg(fin + size_t(nb) * Q * kBlockVoxels + hs[r]) : S();
    }
    const int pc = cube_voxel(i, j, k);
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (is_rest<Q>(q)) continue;
        S* d = st + pc + cube_own<Q>(q);
        if ((cube_own<Q>(q) & 1) == 0) {  // unrolled: a compile-time test
            *reinterpret_cast<W*>(d) = ov[q];
        } else {
            d[0] = lo_of(ov[q]);
            d[1] = hi_of(ov[q]);
        }
    }
#pragma unroll
    for (int r = 0; r < kPer; r++)
        if (hd[r] != 0xffffffffu) st[hd[r] & 0xffffu] = hv[r];
    __syncthreads();

    const int c0 = flag_class(fl.x), c1 = flag_class(fl.y);
    uint32_t  m0 = flag_mask(fl.x), m1 = flag_mask(fl.y);
    if (smissing) {  // a source outside every block is a wall
#pragma unroll
        for (int q = 0; q < Q; q++) {
            if (is_rest<Q>(q)) continue;
            int nv;
            if (bgrid_pull_src<Q>(sconn, i, j, k, q, nv) == NGB_BGRID_NO_BLOCK) m0 |= 1u << q;
            if (bgrid_pull_src<Q>(sconn, i + 1, j, k, q, nv) == NGB_BGRID_NO_BLOCK) m1 |= 1u << q;
        }
    }
    // A voxel that is not bulk is computed beside its partner (from the cube
    // values at its pull positions, which may be unset) but not stored: a
    // pair with one bulk voxel takes the same path as a full pair.
    const bool b0 = c0 == NGB_CELL_BULK, b1 = c1 == NGB_CELL_BULK;
    if (!b0) m0 = 0u;
    if (!b1) m1 = 0u;
    const S* sp = st + pc;
    if (b0 || b1) {
        float2 g[Q];
        if ((m0 | m1) == 0) {
#pragma unroll
            for (int q = 0; q < Q; q++)
                g[q] = PairIO<S>::to_g(is_rest<Q>(q) ? ov[q] : *reinterpret_cast<const W*>(sp + cube_src<Q>(q)), float(L::w(q)));
        } else {
            const uint32_t l0 = m0 ? bgrid_lidbits<Q>(flags, p.mask, sconn, i, j, k, m0) : 0u;
            const uint32_t l1 = m1 ? bgrid_lidbits<Q>(flags, p.mask, sconn, i + 1, j, k, m1) : 0u;
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const int   o = L::opp(q);
                const float w = float(L::w(q));  // w(opp q) == w(q)
                if (is_rest<Q>(q)) {
                    g[q] = PairIO<S>::to_g(ov[q], w);
                } else {
                    const S* a = sp + cube_src<Q>(q);
                    const S* r = sp + cube_own<Q>(o);
                    g[q].x = (m0 >> q) & 1u ? PairIO<S>::to_g1(r[0], w) + ((l0 >> q) & 1u ? p.wall[1][o] : p.wall[0][o])
                                            : PairIO<S>::to_g1(a[0], w);
                    g[q].y = (m1 >> q) & 1u ? PairIO<S>::to_g1(r[1], w) + ((l1 >> q) & 1u ? p.wall[1][o] : p.wall[0][o])
                                            : PairIO<S>::to_g1(a[1], w);
                }
            }
        }
        bgk_shifted<Q, float2, StoreScale<S>::log2>(g, p.omega);
        S* out = fout + size_t(b) * Q * kBlockVoxels + v;
        if (b0 && b1) {
#pragma unroll
            for (int q = 0; q < Q; q++) PairIO<S>::store(out + q * kBlockVoxels, g[q], float(L::w(q)));
        } else if (b0) {
#pragma unroll
            for (int q = 0; q < Q; q++) PairIO<S>::store1(out + q * kBlockVoxels, g[q].x, float(L::w(q)));
        } else {
#pragma unroll
            for (int q = 0; q < Q; q++) PairIO<S>::store1(out + q * kBlockVoxels + 1, g[q].y, float(L::w(q)));
        }
    }
    if (c0 == NGB_CELL_OUTLET) bgrid_outlet<Q, S>(fin, fout, p.mask, p.conn, b, v, i, j, k);
    if (c1 == NGB_CELL_OUTLET) bgrid_outlet<Q, S>(fin, fout, p.mask, p.conn, b, v + 1, i + 1, j, k);
}

template <typename S>
int launch_staged(const ngb_bgrid_desc* d, const void* fin, void* fout, const uint32_t* flags, const BParams<float>& p, cudaStream_t s)
{
    static std::once_flag once;
    static cudaError_t    err = cudaSuccess;
    std::call_once(once, []() {
        err = cudaFuncSetAttribute(bgrid_lbm_staged_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(staged_smem<S>()));
    });
    if (err != cudaSuccess) {
        set_error("bGrid LBM kernel set-up failed: %s", cudaGetErrorString(err));
        return NGB_ERR_CUDA;
    }
    bgrid_lbm_staged_kernel<S><<<d->n_blocks, kStagedThreads, staged_smem<S>(), s>>>(static_cast<const S*>(fin),
                                                                                    static_cast<S*>(fout), flags, p);
    NGB_LAUNCH_CHECK("bgrid_lbm_staged_kernel");
    return NGB_OK;
}

// ---------------------------------------------------------------- drag
template <int Q, typename S>
__global__ void __launch_bounds__(kBlockVoxels) bgrid_drag_kernel(const S* __restrict__ fin, const uint32_t* __restrict__ flags,
                                                                  const uint32_t* __restrict__ mask,
                                                                  const uint32_t* __restrict__ conn, double* partials)
{
    using L = Lattice<Q>;
    const uint32_t b = blockIdx.x;
    const int      v = threadIdx.x, i = v & 7, j = (v >> 3) & 7, k = v >> 6;
    const uint32_t f = __ldg(flags + size_t(b) * kBlockVoxels + v);
    double         F[3] = {0, 0, 0};
    if (flag_class(f) == NGB_CELL_BULK && flag_mask(f)) {
        const uint32_t m = flag_mask(f);
#pragma unroll
        for (int q = 0; q < Q; q++) {
            if (!(m & (1u << q))) continue;
            uint32_t nb;
            int      nv;
            if (!bgrid_valid_ngh(mask, conn, b, i, j, k, -L::cx(q), -L::cy(q), -L::cz(q), nb, nv)) continue;
            if (flag_class(__ldg(flags + size_t(nb) * kBlockVoxels + nv)) != NGB_CELL_BOUNCEBACK) continue;
            const int    o = L::opp(q);
            const double fo = as_f<S>(fin[(size_t(b) * Q + o) * kBlockVoxels + v], L::w(o));
            F[0] += 2.0 * L::cx(o) * fo;
            F[1] += 2.0 * L::cy(o) * fo;
            F[2] += 2.0 * L::cz(o) * fo;
        }
    }
    // fixed-order block reduction: warp butterfly, then warp 0 over the 16 warp sums
    __shared__ double red[3][kBlockVoxels / 32];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double x = F[a];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((v & 31) == 0) red[a][v >> 5] = x;
    }
    __syncthreads();
    if (v < 32) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            double x = v < kBlockVoxels / 32 ? red[a][v] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (v == 0) partials[3 * size_t(b) + a] = x;
        }
    }
}

__global__ void __launch_bounds__(256) drag_final_kernel(const double* __restrict__ partials, int n, double* force)
{
    __shared__ double red[3][256];
    double            s[3] = {0, 0, 0};
    for (int b = threadIdx.x; b < n; b += 256)
        for (int a = 0; a < 3; a++) s[a] += partials[3 * size_t(b) + a];
    for (int a = 0; a < 3; a++) red[a][threadIdx.x] = s[a];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int a = 0; a < 3; a++) red[a][threadIdx.x] += red[a][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3) force[threadIdx.x] = red[threadIdx.x][0];
}

// ---------------------------------------------------------------- geometry
constexpr int kMaxCtrl = 256;
struct GeomParams {
    int    nx, ny, nz, ctrl_dx, n_ctrl;
    double sc[3], r, band, tr, tband;
    double cy[kMaxCtrl], cz[kMaxCtrl];
};

__global__ void sphere_tube_kernel(GeomParams g, uint8_t* active, uint8_t* cls)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const double dx = double(x) - g.sc[0], dy = double(y) - g.sc[1], dz = double(z) - g.sc[2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    const double rs = g.r + g.band;
    bool         act = d2 <= rs * rs;
    const int    seg = x / g.ctrl_dx;
    const double t = double(x - seg * g.ctrl_dx) / double(g.ctrl_dx);
    const double ay = g.cy[seg] + t * (g.cy[seg + 1] - g.cy[seg]);
    const double az = g.cz[seg] + t * (g.cz[seg + 1] - g.cz[seg]);
    const double ty = double(y) - ay, tz = double(z) - az;
    const double rt = g.tr + g.tband;
    act = act || (ty * ty + tz * tz <= rt * rt);
    int c = NGB_CELL_UNDEFINED;
    if (act) {
        if (d2 <= g.r * g.r)
            c = NGB_CELL_BOUNCEBACK;
        else if (x == 0)
            c = NGB_CELL_MOVINGWALL;
        else if (x == g.nx - 1)
            c = NGB_CELL_OUTLET;
        else
            c = NGB_CELL_BULK;
    }
    const size_t cell = size_t(x) + size_t(g.nx) * (size_t(y) + size_t(g.ny) * z);
    if (active) active[cell] = act ? 1 : 0;
    if (cls) cls[cell] = uint8_t(c);
}

int validate(const ngb_bgrid_desc* d)
{
    NGB_CHECK_ARG(d, "desc is NULL");
    NGB_CHECK_ARG(d->n_blocks >= 0, "n_blocks < 0");
    NGB_CHECK_ARG(d->q == 19 || d->q == 27, "q must be 19 or 27 (got %d)", d->q);
    NGB_CHECK_ARG(d->storage >= NGB_STORE_F64 && d->storage <= NGB_STORE_BF16OFF, "bad storage %d", d->storage);
    NGB_CHECK_ARG(d->n_blocks == 0 || (d->origin && d->mask && d->conn), "bGrid arrays must be non-NULL");
    return NGB_OK;
}

}  // namespace

int launch_bgrid_lbm(const ngb_bgrid_desc* d, const void* fin, void* fout, const uint32_t* flags, cudaStream_t s)
{
    if (d->n_blocks == 0) return NGB_OK;
    const bool q19 = d->q == 19;
    if (d->storage == NGB_STORE_F64) {
        BParams<double> p{};
        p.omega = d->omega;
        for (int c = 0; c < 2; c++)
            for (int q = 0; q < 27; q++) p.wall[c][q] = d->wall_term[c][q];
        p.mask = d->mask, p.conn = d->conn;
        const double* a = static_cast<const double*>(fin);
        double*       o = static_cast<double*>(fout);
        if (q19)
            bgrid_lbm_kernel<19, double, true><<<d->n_blocks, kBlockVoxels, 0, s>>>(a, o, flags, p);
        else
            bgrid_lbm_kernel<27, double, true><<<d->n_blocks, kBlockVoxels, 0, s>>>(a, o, flags, p);
        NGB_LAUNCH_CHECK("bgrid_lbm_kernel");
        return NGB_OK;
    }
    BParams<float> p{};
    p.omega = float(d->omega);
    // FP16 values are 2^14 g: the wall terms added to them scale alike
    const float up = d->storage == NGB_STORE_F16OFF ? NGB_F16OFF_SCALE : 1.0f;
    for (int c = 0; c < 2; c++)
        for (int q = 0; q < 27; q++) p.wall[c][q] = float(d->wall_term[c][q]) * up;
    p.mask = d->mask, p.conn = d->conn;
    // D3Q19 with 16-bit storage: the shared-memory staged kernel (measured
    // faster there); FP32 storage and D3Q27: per-direction pull (the staged
    // form measured slower for them)
    if (q19 && d->storage == NGB_STORE_F16OFF) return launch_staged<__half>(d, fin, fout, flags, p, s);
    if (q19 && d->storage == NGB_STORE_BF16OFF) return launch_staged<__nv_bfloat16>(d, fin, fout, flags, p, s);
#define NGB_B(QQ, T) \
    bgrid_lbm_kernel<QQ, T, false><<<d->n_blocks, kBlockVoxels, 0, s>>>(static_cast<const T*>(fin), static_cast<T*>(fout), flags, p)
    switch (d->storage) {
        case NGB_STORE_F32:
            if (q19) NGB_B(19, float); else NGB_B(27, float);
            break;
        case NGB_STORE_F16OFF: NGB_B(27, __half); break;
        default: NGB_B(27, __nv_bfloat16); break;
    }
#undef NGB_B
    NGB_LAUNCH_CHECK("bgrid_lbm_kernel");
    return NGB_OK;
}

}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_bgrid_lbm_step(const ngb_bgrid_desc* d, const void* fin, void* fout, const uint32_t* flags, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(fin && fout && fin != fout && flags, "fin/fout/flags must be non-NULL and fin != fout");
    return launch_bgrid_lbm(d, fin, fout, flags, as_stream(stream));
}

int ngb_bgrid_drag(const ngb_bgrid_desc* d, const void* fin, const uint32_t* flags, double* partials, double* force, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(fin && flags && partials && force, "NULL argument");
    cudaStream_t s = as_stream(stream);
    if (d->n_blocks == 0) {
        NGB_CUDA_TRY(cudaMemsetAsync(force, 0, 3 * sizeof(double), s));
        return NGB_OK;
    }
    const bool q19 = d->q == 19;
#define NGB_D(QQ, T) \
    bgrid_drag_kernel<QQ, T><<<d->n_blocks, kBlockVoxels, 0, s>>>(static_cast<const T*>(fin), flags, d->mask, d->conn, partials)
    switch (d->storage) {
        case NGB_STORE_F64:
            if (q19) NGB_D(19, double); else NGB_D(27, double);
            break;
        case NGB_STORE_F32:
            if (q19) NGB_D(19, float); else NGB_D(27, float);
            break;
        case NGB_STORE_F16OFF:
            if (q19) NGB_D(19, __half); else NGB_D(27, __half);
            break;
        default:
            if (q19) NGB_D(19, __nv_bfloat16); else NGB_D(27, __nv_bfloat16);
            break;
    }
#undef NGB_D
    NGB_LAUNCH_CHECK("bgrid_drag_kernel");
    drag_final_kernel<<<1, 256, 0, s>>>(partials, d->n_blocks, force);
    NGB_LAUNCH_CHECK("drag_final_kernel");
    return NGB_OK;
}

int ngb_geometry_sphere_tube(const ngb_sphere_tube* g, uint8_t* active, uint8_t* cls, void* stream)
{
    NGB_CHECK_ARG(g, "geometry is NULL");
    NGB_CHECK_ARG(g->nx > 0 && g->ny > 0 && g->nz > 0 && g->ny <= 65535 && g->nz <= 65535, "bad dims");
    NGB_CHECK_ARG(g->ctrl_dx > 0, "ctrl_dx must be positive");
    NGB_CHECK_ARG(active || cls, "nothing to write");
    GeomParams p{};
    p.nx = g->nx, p.ny = g->ny, p.nz = g->nz, p.ctrl_dx = g->ctrl_dx;
    p.n_ctrl = g->nx / g->ctrl_dx + 2;
    NGB_CHECK_ARG(p.n_ctrl <= kMaxCtrl, "too many tube control points (nx / ctrl_dx + 2 > %d)", kMaxCtrl);
    for (int a = 0; a < 3; a++) p.sc[a] = g->sphere_c[a];
    p.r = g->sphere_r, p.band = g->band, p.tr = g->tube_r, p.tband = g->tube_band;
    std::mt19937_64 rng(g->seed);
    auto            u01 = [&]() { return double(rng() >> 11) * (1.0 / 9007199254740992.0); };
    for (int c = 0; c < p.n_ctrl; c++) {
        p.cy[c] = g->tube_c[0] + g->amplitude * (2.0 * u01() - 1.0);
        p.cz[c] = g->tube_c[1] + g->amplitude * (2.0 * u01() - 1.0);
    }
    sphere_tube_kernel<<<dim3((g->nx + 127) / 128, g->ny, g->nz), 128, 0, as_stream(stream)>>>(p, active, cls);
    NGB_LAUNCH_CHECK("sphere_tube_kernel");
    return NGB_OK;
}

}  // extern "C"
