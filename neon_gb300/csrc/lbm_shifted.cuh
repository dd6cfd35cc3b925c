// Dense LBM pull stream-collide, FP32 compute on equilibrium-shifted values
// (g = f - w), one cell per thread, x fastest: each population plane is read
// with one coalesced (+-1-element shifted) row access per warp and written with
// one aligned row access, so every population element crosses HBM once per
// step. Plane offsets depend only on kernel parameters (warp-uniform).
// The BGK helper also has a float2 form for Blackwell's packed FP32x2
// instructions (fma/add/mul .f32x2), used where two cells share a thread.
//
// The arithmetic is an explicit sequence of IEEE operations (this file is
// compiled with --fmad=false; every fused multiply-add is written out), so a
// CPU restatement using std::fmaf at the same places reproduces it bit for bit:
//   drho = sum_q g_q (q ascending); j_a = sum_{c_a>0} g - sum_{c_a<0} g
//   rho = 1 + drho; inv = 1 / rho; u = j * inv
//   usq = fma(uz, uz, fma(uy, uy, ux*ux)); rus = rho * (1.5 * usq); base = drho - rus
//   u3 = 3 u; per weight class: wr = w rho, wb = w base
//   per q: t = c . u3 (adds in x, y, z order); a = fma(0.5 t, t, t)
//          eqg = fma(wr, a, wb); g' = fma(omega, eqg - g, g)
#pragma once
#include "lbm_kernels.cuh"

namespace ngb {

// ------------------------------------------------------------------ packed FP32 helpers
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float  add2(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float  sub2(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float  mul2(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float  fma2(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <typename V>
__device__ __forceinline__ V splat(float a);
template <>
__device__ __forceinline__ float2 splat<float2>(float a) { return make_float2(a, a); }
template <>
__device__ __forceinline__ float splat<float>(float a) { return a; }
__device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float  neg(float a) { return -a; }
__device__ __forceinline__ float2 recip(float2 a) { return make_float2(1.f / a.x, 1.f / a.y); }
__device__ __forceinline__ float  recip(float a) { return 1.f / a; }

// ------------------------------------------------------------------ storage access in pairs
template <typename S>
struct PairIO;

template <>
struct PairIO<float> {
    static constexpr bool kStochastic = false;
    using Word = float2;
    __device__ __forceinline__ static float ldg1(const char* p, float w) { return __ldg(reinterpret_cast<const float*>(p)) - w; }
    __device__ __forceinline__ static Word load(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
    // (a.hi, b.lo)
    __device__ __forceinline__ static Word mid(Word a, Word b) { return make_float2(a.y, b.x); }
    __device__ __forceinline__ static float2 to_g(Word v, float w) { return make_float2(v.x - w, v.y - w); }
    __device__ __forceinline__ static float  to_g1(float v, float w) { return v - w; }
    __device__ __forceinline__ static void   store(float* p, float2 g, float w)
    {
        *reinterpret_cast<float2*>(p) = make_float2(w + g.x, w + g.y);
    }
    __device__ __forceinline__ static void store1(float* p, float g, float w) { *p = w + g; }
};

template <>
struct PairIO<__half> {
    static constexpr bool kStochastic = false;
    using Word = __half2;
    __device__ __forceinline__ static float ldg1(const char* p, float) { return __half2float(__ldg(reinterpret_cast<const __half*>(p))); }
    __device__ __forceinline__ static Word load(const __half* p) { return __ldg(reinterpret_cast<const __half2*>(p)); }
    __device__ __forceinline__ static Word mid(Word a, Word b) { return __halves2half2(__high2half(a), __low2half(b)); }
    __device__ __forceinline__ static float2 to_g(Word v, float) { return __half22float2(v); }
    __device__ __forceinline__ static float  to_g1(__half v, float) { return __half2float(v); }
    __device__ __forceinline__ static void   store(__half* p, float2 g, float)
    {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(g.x, g.y);
    }
    __device__ __forceinline__ static void store1(__half* p, float g, float) { *p = __float2half_rn(g); }
};

template <>
struct PairIO<__nv_bfloat16> {
    static constexpr bool kStochastic = false;
    using Word = __nv_bfloat162;
    __device__ __forceinline__ static float ldg1(const char* p, float)
    {
        return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p)));
    }
    __device__ __forceinline__ static Word load(const __nv_bfloat16* p)
    {
        return __ldg(reinterpret_cast<const __nv_bfloat162*>(p));
    }
    __device__ __forceinline__ static Word mid(Word a, Word b) { return __halves2bfloat162(__high2bfloat16(a), __low2bfloat16(b)); }
    __device__ __forceinline__ static float2 to_g(Word v, float) { return __bfloat1622float2(v); }
    __device__ __forceinline__ static float  to_g1(__nv_bfloat16 v, float) { return __bfloat162float(v); }
    __device__ __forceinline__ static void   store(__nv_bfloat16* p, float2 g, float)
    {
        *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(g.x, g.y);
    }
    __device__ __forceinline__ static void store1(__nv_bfloat16* p, float g, float) { *p = __float2bfloat16_rn(g); }
};

// FP16 stores with stochastic rounding, by the hardware's stochastic-rounding
// conversion (cvt.rs): a 13-bit random number r in [0, 8192) is added, in
// units of 2^-13 of the result's ulp, to the magnitude, which is then
// truncated, so the value rounds up in magnitude with probability = its
// remainder / ulp (FP16 subnormal results included). One 32-bit word carries
// the bits of a pair: bits 0-12 for the low half, 16-28 for the high half.
__device__ __forceinline__ uint32_t f16x2_sr(float lo, float hi, uint32_t rbits)
{
    uint32_t w;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(w) : "f"(hi), "f"(lo), "r"(rbits));
    return w;
}
__device__ __forceinline__ __half f16_sr(float v, uint32_t r)
{
    return __ushort_as_half(static_cast<unsigned short>(f16x2_sr(v, 0.f, r) & 0xffffu));
}

template <>
struct PairIO<f16sr_t> {
    static constexpr bool kStochastic = true;
    __device__ __forceinline__ static float ldg1(const char* p, float) { return __half2float(__ldg(reinterpret_cast<const __half*>(p))); }
    __device__ __forceinline__ static void  store1(f16sr_t* p, float g, float, uint32_t r)
    {
        *reinterpret_cast<__half*>(p) = f16_sr(g, r);
    }
};

// Store of one computed value (the dither bits r are used by stochastic storage only).
template <typename S>
__device__ __forceinline__ void store_g(S* p, float g, float w, uint32_t r)
{
    if constexpr (PairIO<S>::kStochastic)
        PairIO<S>::store1(p, g, w, r);
    else
        PairIO<S>::store1(p, g, w);
}
// 13 dither bits of population q of `cell` (stochastic storage only)
template <typename S>
__device__ __forceinline__ uint32_t dither_of(uint32_t h, int q, int64_t cell)
{
    if constexpr (PairIO<S>::kStochastic) {
        const uint32_t hq = dither_word(h, q);
        return (cell & 1) ? dither_hi(hq) : dither_lo(hq);
    } else {
        return 0u;
    }
}
template <typename S>
__device__ __forceinline__ uint32_t dither_base(int64_t cell, uint32_t seed)
{
    if constexpr (PairIO<S>::kStochastic)
        return dither_hash(cell, seed);
    else
        return 0u;
}

// Byte offsets, relative to a cell's own element of plane 0, of each
// direction's pull source (q * stride - c_q . (1, nx, nx ny)) and of each of
// the cell's own planes (q * stride). They depend only on the grid, so the
// host computes them once: recomputing them per thread in 64-bit integer
// arithmetic was the largest instruction class of the 16-bit kernels.
struct DirOffsets {
    int64_t pull[27];
    int64_t own[27];
};

// Scalar pull of one cell's populations as g (wall rule included): one 64-bit
// address add per load.
template <int Q, typename S>
__device__ __forceinline__ void pull_one(const S* __restrict__ fin, int64_t cell, uint32_t mask, uint32_t lidbits,
                                         const DenseParams<float>& p, const DirOffsets& o, float* g)
{
    using L = Lattice<Q>;
    const char* P = reinterpret_cast<const char*>(fin + cell);
    if (mask == 0) {
#pragma unroll
        for (int q = 0; q < Q; q++) g[q] = PairIO<S>::ldg1(P + o.pull[q], float(L::w(q)));
        return;
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (mask & (1u << q)) {
            const int   oq = L::opp(q);
            const float wt = (lidbits & (1u << q)) ? p.wall[1][oq] : p.wall[0][oq];
            g[q] = PairIO<S>::ldg1(P + o.own[oq], float(L::w(oq))) + wt;
        } else {
            g[q] = PairIO<S>::ldg1(P + o.pull[q], float(L::w(q)));
        }
    }
}

template <int Q>
struct WeightClass;
template <>
struct WeightClass<19> {
    static constexpr int n = 3;
    __host__ __device__ static constexpr int of(int q) { return q == 9 ? 0 : ((q % 10) < 3 ? 1 : 2); }
    __host__ __device__ static constexpr double w(int k) { return k == 0 ? 1. / 3. : (k == 1 ? 1. / 18. : 1. / 36.); }
};
template <>
struct WeightClass<27> {
    static constexpr int n = 4;
    __host__ __device__ static constexpr int of(int q)
    {
        return (Lattice<27>::cx(q) != 0) + (Lattice<27>::cy(q) != 0) + (Lattice<27>::cz(q) != 0);
    }
    __host__ __device__ static constexpr double w(int k)
    {
        return k == 0 ? 8. / 27. : (k == 1 ? 2. / 27. : (k == 2 ? 1. / 54. : 1. / 216.));
    }
};

// t = c_q . u3 with adds in x, y, z order (first non-zero component starts the sum).
template <int Q, typename V>
__device__ __forceinline__ V cdot(int q, V u3x, V u3y, V u3z)
{
    using L = Lattice<Q>;
    V          t = splat<V>(0.f);
    bool       started = false;
    const int  c[3] = {L::cx(q), L::cy(q), L::cz(q)};
    const V    u[3] = {u3x, u3y, u3z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (c[a] == 0) continue;
        if (!started) {
            t = c[a] > 0 ? u[a] : neg(u[a]);
            started = true;
        } else {
            t = c[a] > 0 ? add2(t, u[a]) : sub2(t, u[a]);
        }
    }
    return t;
}

template <int Q, typename V, int SH>
__device__ __forceinline__ void bgk_relax(V (&g)[Q], V drho, V rho, V ux, V uy, V uz, float omega);

// Shifted BGK on V = float (one cell) or float2 (a cell pair): g -> g' in place.
// SH: the values are G = 2^SH g (FP16 storage). Every quantity of the
// sequence below is then exactly 2^SH times its unscaled value (power-of-two
// scaling commutes with rounding) once drho and 1/rho are taken back by
// 2^-SH and the weights enter as 2^SH w: the stored result is the same
// rounding of the same number.
template <int Q, typename V, int SH = 0>
__device__ __forceinline__ void bgk_shifted(V (&g)[Q], float omega)
{
    constexpr float kUp = float(1u << SH), kDown = 1.0f / kUp;
    using L = Lattice<Q>;
    V drho = g[0];
#pragma unroll
    for (int q = 1; q < Q; q++) drho = add2(drho, g[q]);
    V    jp[3] = {splat<V>(0.f), splat<V>(0.f), splat<V>(0.f)}, jm[3] = {splat<V>(0.f), splat<V>(0.f), splat<V>(0.f)};
    bool sp[3] = {false, false, false}, sm[3] = {false, false, false};
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int c[3] = {L::cx(q), L::cy(q), L::cz(q)};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (c[a] > 0) {
                jp[a] = sp[a] ? add2(jp[a], g[q]) : g[q];
                sp[a] = true;
            } else if (c[a] < 0) {
                jm[a] = sm[a] ? add2(jm[a], g[q]) : g[q];
                sm[a] = true;
            }
        }
    }
    const V jx = sub2(jp[0], jm[0]), jy = sub2(jp[1], jm[1]), jz = sub2(jp[2], jm[2]);
    if constexpr (SH != 0) drho = mul2(drho, splat<V>(kDown));
    const V rho = add2(splat<V>(1.f), drho);
    V       inv = recip(rho);
    if constexpr (SH != 0) inv = mul2(inv, splat<V>(kDown));
    const V ux = mul2(jx, inv), uy = mul2(jy, inv), uz = mul2(jz, inv);
    bgk_relax<Q, V, SH>(g, drho, rho, ux, uy, uz, omega);
}

// The relaxation part of the shifted BGK: g <- g + omega (eq_g(drho, u) - g)
// with the values of g held as 2^SH g; drho, rho and u are unscaled.
template <int Q, typename V, int SH>
__device__ __forceinline__ void bgk_relax(V (&g)[Q], V drho, V rho, V ux, V uy, V uz, float omega)
{
    constexpr float kUp = float(1u << SH);
    const V usq = fma2(uz, uz, fma2(uy, uy, mul2(ux, ux)));
    const V rus = mul2(rho, mul2(splat<V>(1.5f), usq));
    const V base = sub2(drho, rus);
    const V u3x = mul2(splat<V>(3.f), ux), u3y = mul2(splat<V>(3.f), uy), u3z = mul2(splat<V>(3.f), uz);
    V       wr[WeightClass<Q>::n], wb[WeightClass<Q>::n];
#pragma unroll
    for (int k = 0; k < WeightClass<Q>::n; k++) {
        const float wk = float(WeightClass<Q>::w(k)) * kUp;  // exact
        wr[k] = mul2(splat<V>(wk), rho);
        wb[k] = mul2(splat<V>(wk), base);
    }
    const V om = splat<V>(omega);
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int k = WeightClass<Q>::of(q);
        const V   t = cdot<Q, V>(q, u3x, u3y, u3z);
        const V   a = fma2(mul2(splat<V>(0.5f), t), t, t);
        const V   eqg = fma2(wr[k], a, wb[k]);
        g[q] = fma2(om, sub2(eqg, g[q]), g[q]);
    }
}

// Zou-He node (D3Q19) in the shifted FP32 form, on its pulled populations
// (the unknown ones are overwritten): M and K of the known populations (float
// adds, q ascending, taken back to unscaled values), mk = M + (K + K);
// PRESSURE: drho = rho_b - 1, rho = 1 + drho, s u_a = (drho - mk) / rho;
// VELOCITY: u = u_b, un = s u_a, drho = (mk + un) / (1 - un), rho = 1 + drho;
// unknowns g_q = fma((2 w_q) rho, c_q . 3u, g_opp(q)) (f_q - f_opp(q) =
// eq_q - eq_opp(q) = 6 w_q rho c_q . u); then the shifted relaxation.
template <int Q, typename S>
__device__ __forceinline__ void zouhe_node_shifted(float (&g)[Q], int cls, int x, int y, int z, const DenseParams<float>& p)
{
    using L = Lattice<Q>;
    constexpr int   SH = StoreScale<S>::log2;
    constexpr float kUp = float(1u << SH), kDown = 1.0f / kUp;
    int             a, s;
    zouhe_normal(x, y, z, p.nx, p.ny, p.nz, a, s);
    float M = 0.f, K = 0.f;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int ca = lattice_c<Q>(q, a);
        if (ca == 0) M = M + g[q];
        else if (ca * s == -1) K = K + g[q];
    }
    if constexpr (SH != 0) {
        M = M * kDown;
        K = K * kDown;
    }
    const float mk = M + (K + K);
    float       u[3] = {0.f, 0.f, 0.f}, drho, rho;
    if (cls == NGB_CELL_PRESSURE) {
        drho = p.zh_rho;
        rho = 1.f + drho;
        u[a] = float(s) * ((drho - mk) / rho);
    } else {
        for (int d = 0; d < 3; d++) u[d] = p.zh_u[d];
        const float un = float(s) * u[a];
        drho = (mk + un) / (1.f - un);
        rho = 1.f + drho;
    }
    const float u3x = 3.f * u[0], u3y = 3.f * u[1], u3z = 3.f * u[2];
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (lattice_c<Q>(q, a) * s != 1) continue;
        const float coef = ((2.f * float(L::w(q))) * kUp) * rho;
        g[q] = __fmaf_rn(coef, cdot<Q, float>(q, u3x, u3y, u3z), g[L::opp(q)]);
    }
    bgk_relax<Q, float, SH>(g, drho, rho, u[0], u[1], u[2], p.omega);
}

// One cell (x, y, z): classification, pull, collision, stores.
template <int Q, typename S>
__device__ __forceinline__ void lbm_cell(const S* __restrict__ fin, S* __restrict__ fout, const uint32_t* __restrict__ flags,
                                         const DenseParams<float>& p, const DirOffsets& o, int x, int y, int z)
{
    using L = Lattice<Q>;
    const int64_t cell = x + int64_t(p.nx) * (y + int64_t(p.ny) * z);
    uint32_t      mask, lidbits;
    const int     cls = cell_setup<Q>(p, flags, x, y, z, cell, mask, lidbits);
    if (cls == NGB_CELL_OUTLET) {
        outlet_copy<Q>(fin, fout, p.stride, cell, x, flags);
        return;
    }
    const bool zh = is_zouhe_class(cls);
    if (cls != NGB_CELL_BULK && !(Q == 19 && zh)) return;
    float g[Q];
    // a Zou-He node's unknown directions come from outside the box: masked,
    // so the pull reads the node's own opposite populations there (replaced below)
    pull_one<Q, S>(fin, cell, mask, lidbits, p, o, g);
    if (zh)
        zouhe_node_shifted<Q, S>(g, cls, x, y, z, p);
    else
        bgk_shifted<Q, float, StoreScale<S>::log2>(g, p.omega);
    const uint32_t h = dither_base<S>(cell, p.seed);
    char*          D = reinterpret_cast<char*>(fout + cell);
#pragma unroll
    for (int q = 0; q < Q; q++) store_g<S>(reinterpret_cast<S*>(D + o.own[q]), g[q], float(L::w(q)), dither_of<S>(h, q, cell));
}

// One cell per thread, every cell of the grid.
template <int Q, typename S>
__global__ void __launch_bounds__(kLbmBlockX) lbm_dense_single_kernel(const S* __restrict__ fin, S* __restrict__ fout,
                                                                     const uint32_t* __restrict__ flags, DenseParams<float> p,
                                                                     const __grid_constant__ DirOffsets o)
{
    const int x = blockIdx.x * kLbmBlockX + threadIdx.x;
    if (x >= p.nx) return;
    lbm_cell<Q, S>(fin, fout, flags, p, o, x, blockIdx.y, blockIdx.z);
}

// Analytic cavity, split by the walls a cell can see. The core covers
// x in [1, nx-2], y in [2, ny-3], z in [2, nz-3] (threads on x from 0, so
// warps keep the alignment of the rows): every cell is bulk and its
// only wall sources are the resting x walls of the cells x = 1 (directions
// with c_x = +1) and x = nx-2 (c_x = -1), which read the cell's own opposite
// population plus the bounce-back wall term. Warps without such a cell take
// the plain pull (no classification at all); the two warps of a row that
// hold one select the source per lane, so no warp diverges. The shell kernel
// below takes the remaining bulk cells (y or z next to a wall).
template <int Q, typename S>
__global__ void __launch_bounds__(kLbmBlockX) lbm_box_core_kernel(const S* __restrict__ fin, S* __restrict__ fout,
                                                                 DenseParams<float> p, const __grid_constant__ DirOffsets o)
{
    using L = Lattice<Q>;
    const int      x = blockIdx.x * kLbmBlockX + threadIdx.x;  // rows stay 128-byte aligned: x = 0 is a dead lane
    const int      y = 2 + blockIdx.y, z = 2 + blockIdx.z;
    const bool     live = x >= 1 && x <= p.nx - 2;
    const bool     lo = x == 1, hi = x == p.nx - 2;
    const unsigned edge_warp = __ballot_sync(0xffffffffu, live && (lo || hi));
    if (!live) return;
    const int64_t cell = x + int64_t(p.nx) * (y + int64_t(p.ny) * z);
    const char*   P = reinterpret_cast<const char*>(fin + cell);
    float         g[Q];
    if (edge_warp == 0) {
#pragma unroll
        for (int q = 0; q < Q; q++) g[q] = PairIO<S>::ldg1(P + o.pull[q], float(L::w(q)));
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int cx = L::cx(q);
            if (cx == 0) {
                g[q] = PairIO<S>::ldg1(P + o.pull[q], float(L::w(q)));
            } else {
                const int     oq = L::opp(q);
                const bool    wall = cx > 0 ? lo : hi;
                const int64_t off = wall ? o.own[oq] : o.pull[q];
                const float   wt = wall ? p.wall[0][oq] : 0.f;
                const float   w = float(wall ? L::w(oq) : L::w(q));
                const float   v = PairIO<S>::ldg1(P + off, w);
                g[q] = wall ? v + wt : v;
            }
        }
    }
    bgk_shifted<Q, float, StoreScale<S>::log2>(g, p.omega);
    const uint32_t h = dither_base<S>(cell, p.seed);
    char*          D = reinterpret_cast<char*>(fout + cell);
#pragma unroll
    for (int q = 0; q < Q; q++) store_g<S>(reinterpret_cast<S*>(D + o.own[q]), g[q], float(L::w(q)), dither_of<S>(h, q, cell));
}

// ------------------------------------------------------------------ x-pair core kernel (16-bit storage)
// The core region of the analytic cavity with one thread per aligned pair of
// cells (2t, 2t+1) of a row: every population plane is read with one 32-bit
// load per thread (128 bytes per warp instruction instead of 64) and written
// with one 32-bit store. A direction with c_x = 0 reads its pair directly; for
// c_x = +1 the pair (2t-1, 2t) is the high half of the left neighbour's word
// (warp shuffle) and the low half of the own word, for c_x = -1 the pair
// (2t+1, 2t+2) is the own high half and the right neighbour's low half; the
// first / last lane of a warp loads the aligned word beyond the warp's ends.
// The collision runs on FP32x2 pairs (per lane the scalar sequence, so the
// stored bits equal the one-cell kernels'). The pairs holding x = 1 and
// x = nx-2 take the resting-wall bounce-back per half; x = 0 and x = nx-1 are
// wall nodes and are not written. Warps that hold such a pair or an idle lane
// take a separate path; the rest of the row runs without any per-direction
// test. A thread walks ZC planes in z with the next plane's words loaded
// before the current plane's collision (ZC = 1: one plane, no prefetch).
// Requires nx even (rows start on a word).
constexpr int kPairBlock = 64;

__device__ __forceinline__ uint32_t ldg_u32(const char* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }

template <typename S>
struct PairBits;
template <>
struct PairBits<__half> {
    __device__ __forceinline__ static float2 to_g(uint32_t w)
    {
        __half2 h;
        memcpy(&h, &w, 4);
        return __half22float2(h);
    }
    __device__ __forceinline__ static uint32_t from_g(float2 g)
    {
        const __half2 h = __floats2half2_rn(g.x, g.y);
        uint32_t      w;
        memcpy(&w, &h, 4);
        return w;
    }
};
template <>
struct PairBits<__nv_bfloat16> {
    __device__ __forceinline__ static float2 to_g(uint32_t w)
    {
        __nv_bfloat162 h;
        memcpy(&h, &w, 4);
        return __bfloat1622float2(h);
    }
    __device__ __forceinline__ static uint32_t from_g(float2 g)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(g.x, g.y);
        uint32_t             w;
        memcpy(&w, &h, 4);
        return w;
    }
};

template <>
struct PairBits<f16sr_t> {
    __device__ __forceinline__ static float2 to_g(uint32_t w) { return PairBits<__half>::to_g(w); }
    // the pair's cells are even (lo) and odd (hi): their dither bits come from one word
    __device__ __forceinline__ static uint32_t from_g_sr(float2 g, uint32_t hq) { return f16x2_sr(g.x, g.y, hq); }
};

// Plane walk and register cap of the pair kernel per storage: FP16 with
// stochastic rounding spends more instructions per pair, so it hides the
// load latency with the prefetch of the next plane (16 planes per thread,
// up to 128 registers); the other 16-bit forms run one plane per thread at
// 64 registers (32 warps per SM). Measured at 384^3, same process.
template <typename S, int Q = 19>
struct PairWalk {
    static constexpr int planes = 1, min_ctas = 16;
};
template <>
struct PairWalk<f16sr_t, 19> {
    static constexpr int planes = 16, min_ctas = 8;
};
// D3Q27: 27 pulled values per cell pair, one plane per thread, up to 128 registers
template <typename S>
struct PairWalk<S, 27> {
    static constexpr int planes = 1, min_ctas = 8;
};

// Directions with c_x = +1 (and as many with -1) of a lattice.
template <int Q>
__host__ __device__ constexpr int x_plus_count()
{
    int n = 0;
    for (int q = 0; q < Q; q++) n += Lattice<Q>::cx(q) > 0 ? 1 : 0;
    return n;
}

// The 32-bit words one pair pulls along every direction (w), and for the
// first / last lane of a warp the word beyond the warp's end along each
// c_x = +1 (xa) / -1 (xb) direction; for the pairs at x = 1 / x = nx - 2 that
// slot holds the pair's own word of the opposite direction (bounce-back).
template <int Q>
__device__ __forceinline__ void pair_fetch(const char* P, const DirOffsets& o, int lane, bool first, bool last, uint32_t (&w)[Q],
                                           uint32_t (&xa)[x_plus_count<Q>()], uint32_t (&xb)[x_plus_count<Q>()])
{
    using L = Lattice<Q>;
    int ia = 0, ib = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int   cx = L::cx(q);
        const char* src = P + o.pull[q];  // the pull source of the pair's first cell
        if (cx == 0) {
            w[q] = ldg_u32(src);
        } else if (cx > 0) {
            w[q] = ldg_u32(src + 2);
            if (lane == 0) xa[ia] = ldg_u32(first ? P + o.own[L::opp(q)] : src - 2);
            ia++;
        } else {
            w[q] = ldg_u32(src - 2);
            if (last || lane == 31) xb[ib] = ldg_u32(last ? P + o.own[L::opp(q)] : src + 2);
            ib++;
        }
    }
}

// Words -> the pair's pulled values as FP32 pairs (shuffles, byte permutes,
// bounce-back at the row ends).
template <int Q, typename S, bool EDGE>
__device__ __forceinline__ void pair_unpack(const uint32_t (&w)[Q], const uint32_t (&xa)[x_plus_count<Q>()],
                                            const uint32_t (&xb)[x_plus_count<Q>()], int lane, bool first, bool last,
                                            const DenseParams<float>& p, float2 (&g)[Q])
{
    using L = Lattice<Q>;
    int ia = 0, ib = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int cx = L::cx(q);
        if (cx == 0) {
            g[q] = PairBits<S>::to_g(w[q]);
        } else if (cx > 0) {
            uint32_t left = __shfl_up_sync(0xffffffffu, w[q], 1);
            if (lane == 0) left = xa[ia];
            g[q] = PairBits<S>::to_g(__byte_perm(left, w[q], 0x5432));
            if (EDGE && first) g[q].y = PairBits<S>::to_g(xa[ia]).y + p.wall[0][L::opp(q)];
            ia++;
        } else {
            uint32_t right = __shfl_down_sync(0xffffffffu, w[q], 1);
            if (lane == 31) right = xb[ib];
            g[q] = PairBits<S>::to_g(__byte_perm(w[q], right, 0x5432));
            if (EDGE && last) g[q].x = PairBits<S>::to_g(xb[ib]).x + p.wall[0][L::opp(q)];
            ib++;
        }
    }
}

template <int Q, typename S, bool EDGE>
__device__ __forceinline__ void pair_store(char* D, const DirOffsets& o, const float2 (&g)[Q], uint32_t h, bool first, bool last)
{
#pragma unroll
    for (int q = 0; q < Q; q++) {
        uint32_t w;
        if constexpr (PairIO<S>::kStochastic)
            w = PairBits<S>::from_g_sr(g[q], dither_word(h, q));
        else
            w = PairBits<S>::from_g(g[q]);
        if (!EDGE || !(first || last))
            *reinterpret_cast<unsigned int*>(D + o.own[q]) = w;
        else if (first)  // x = 0 is a wall node
            *reinterpret_cast<unsigned short*>(D + o.own[q] + 2) = static_cast<unsigned short>(w >> 16);
        else  // x = nx - 1 is a wall node
            *reinterpret_cast<unsigned short*>(D + o.own[q]) = static_cast<unsigned short>(w & 0xffffu);
    }
}

// One pair's column of planes z0 .. z1-1.
template <int Q, typename S, bool EDGE>
__device__ __forceinline__ void pair_column(const S* __restrict__ fin, S* __restrict__ fout, const DenseParams<float>& p,
                                            const DirOffsets& o, int64_t cell, int z0, int z1, int lane, bool live, bool first,
                                            bool last)
{
    const int64_t zs = int64_t(p.nx) * p.ny * int64_t(sizeof(S));  // bytes per plane
    const char*   P = reinterpret_cast<const char*>(fin + cell);
    char*         D = reinterpret_cast<char*>(fout + cell);
    constexpr int kX = x_plus_count<Q>();
    uint32_t      w[Q], xa[kX], xb[kX];
#pragma unroll
    for (int e = 0; e < kX; e++) xa[e] = 0u, xb[e] = 0u;
    pair_fetch<Q>(P, o, lane, first, last, w, xa, xb);
    for (int z = z0; z < z1; z++) {
        float2 g[Q];
        pair_unpack<Q, S, EDGE>(w, xa, xb, lane, first, last, p, g);
        if (z + 1 < z1) pair_fetch<Q>(P + zs, o, lane, first, last, w, xa, xb);
        bgk_shifted<Q, float2, StoreScale<S>::log2>(g, p.omega);
        if (!EDGE || live) pair_store<Q, S, EDGE>(D, o, g, dither_base<S>(cell, p.seed), first, last);
        P += zs;
        D += zs;
        cell += int64_t(p.nx) * p.ny;
    }
}

template <int Q, typename S>
__global__ void __launch_bounds__(kPairBlock, PairWalk<S, Q>::min_ctas)
    lbm_box_core_pair_kernel(const S* __restrict__ fin, S* __restrict__ fout, DenseParams<float> p, const __grid_constant__ DirOffsets o)
{
    constexpr int  ZC = PairWalk<S, Q>::planes;
    const int      np = p.nx >> 1;  // pairs per row
    const int      t = blockIdx.x * kPairBlock + threadIdx.x, lane = threadIdx.x & 31;
    const bool     live = t < np;
    const int      tp = live ? t : np - 1;  // idle lanes read the last pair (in the row, results unused)
    const int      y = 2 + blockIdx.y, z0 = 2 + blockIdx.z * ZC, z1 = min(z0 + ZC, p.nz - 2);
    const bool     first = tp == 0, last = tp == np - 1;  // the pairs holding x = 1 and x = nx - 2
    const unsigned edge = __ballot_sync(0xffffffffu, !live || first || last);
    const int64_t  cell = 2 * int64_t(tp) + int64_t(p.nx) * (y + int64_t(p.ny) * z0);
    if (edge)
        pair_column<Q, S, true>(fin, fout, p, o, cell, z0, z1, lane, live, first, last);
    else
        pair_column<Q, S, false>(fin, fout, p, o, cell, z0, z1, lane, true, false, false);
}

// The rest of the analytic cavity's bulk cells: the planes z = 1 and
// z = nz-2 (y in [1, ny-2]) and the rows y = 1 and y = ny-2 of the planes
// z in [2, nz-3], x in [1, nx-2]; blockIdx.y enumerates these rows.
template <int Q, typename S>
__global__ void __launch_bounds__(kLbmBlockX) lbm_box_shell_kernel(const S* __restrict__ fin, S* __restrict__ fout,
                                                                  DenseParams<float> p, const __grid_constant__ DirOffsets o)
{
    const int x = blockIdx.x * kLbmBlockX + threadIdx.x;
    if (x < 1 || x > p.nx - 2) return;
    const int r = blockIdx.y, ry = p.ny - 2, rz = p.nz - 4;
    int       y, z;
    if (r < 2 * ry) {
        z = r < ry ? 1 : p.nz - 2;
        y = 1 + (r < ry ? r : r - ry);
    } else {
        const int t = r - 2 * ry;
        y = t < rz ? 1 : p.ny - 2;
        z = 2 + (t < rz ? t : t - rz);
    }
    lbm_cell<Q, S>(fin, fout, nullptr, p, o, x, y, z);
}

}  // namespace ngb
