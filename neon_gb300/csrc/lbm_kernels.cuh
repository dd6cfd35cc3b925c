// Dense single-partition LBM pull stream-collide kernels (D3Q19 / D3Q27).
//
// Layout: population (x, y, z, q) at x + nx*(y + ny*z) + q*stride (SoA planes).
// One thread per cell, x fastest: every population plane is read with one
// coalesced (at most +-1-element shifted) row access per warp and written
// with one aligned row access, so each population element crosses HBM once
// per step: 2 * Q * sizeof(storage) bytes per lattice update.
#pragma once
#include "common.cuh"

namespace ngb {

constexpr int kLbmBlockX = 128;

template <typename C>
struct DenseParams {
    int32_t nx, ny, nz;
    int32_t box;      // 1: analytic cavity classification
    int64_t stride;   // elements between planes
    C       omega;
    C       wall[2][27];  // wall term by wall class (bounce-back, moving wall), compute type
    C        zh_rho;      // Zou-He PRESSURE nodes: rho (FP64 compute) or rho - 1 (FP32 shifted compute)
    C        zh_u[3];     // Zou-He VELOCITY nodes: u
    uint32_t seed;        // F16SR: dither seed of this step
};

// Inward normal of a Zou-He node: the first box face it lies on, in the order
// x = 0, x = nx-1, y = 0, y = ny-1, z = 0, z = nz-1 (axis a, sign s).
__host__ __device__ inline void zouhe_normal(int x, int y, int z, int nx, int ny, int nz, int& a, int& s)
{
    if (x == 0) a = 0, s = 1;
    else if (x == nx - 1) a = 0, s = -1;
    else if (y == 0) a = 1, s = 1;
    else if (y == ny - 1) a = 1, s = -1;
    else if (z == 0) a = 2, s = 1;
    else a = 2, s = -1;
}
template <int Q>
__host__ __device__ constexpr int lattice_c(int q, int a)
{
    return a == 0 ? Lattice<Q>::cx(q) : (a == 1 ? Lattice<Q>::cy(q) : Lattice<Q>::cz(q));
}

// Classification and wall mask of cell (x,y,z) for the analytic lid-driven
// cavity (RunCavityTwoPop.cu:208-224 + LbmTools.h:327-376): faces are walls,
// y = ny-1 is the moving lid; for interior cells bit q is set iff x - c_q is
// on a face. `lidbits` gets bit q set iff that face node is on the lid.
template <int Q>
__device__ __forceinline__ int box_classify(int x, int y, int z, int nx, int ny, int nz, uint32_t& mask, uint32_t& lidbits)
{
    mask = 0;
    lidbits = 0;
    if (y == ny - 1) return NGB_CELL_MOVINGWALL;
    if (x == 0 || x == nx - 1 || y == 0 || z == 0 || z == nz - 1) return NGB_CELL_BOUNCEBACK;
    const bool xl = x == 1, xh = x == nx - 2, yl = y == 1, yh = y == ny - 2, zl = z == 1, zh = z == nz - 2;
    if (!(xl | xh | yl | yh | zl | zh)) return NGB_CELL_BULK;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int  cx = Lattice<Q>::cx(q), cy = Lattice<Q>::cy(q), cz = Lattice<Q>::cz(q);
        const bool w = (cx > 0 && xl) || (cx < 0 && xh) || (cy > 0 && yl) || (cy < 0 && yh) || (cz > 0 && zl) || (cz < 0 && zh);
        if (w) mask |= 1u << q;
        if (cy < 0 && yh) lidbits |= 1u << q;
    }
    return NGB_CELL_BULK;
}

// Wall class of the pull source of direction q of a bulk cell in flags mode.
__device__ __forceinline__ int source_class(const uint32_t* __restrict__ flags, int64_t src)
{
    return flag_class(__ldg(flags + src));
}

// Common cell prologue: returns the class; for bulk cells fills mask and
// per-direction wall class bits (bit q set -> the source is a moving wall).
template <int Q, typename C>
__device__ __forceinline__ int cell_setup(const DenseParams<C>& p, const uint32_t* __restrict__ flags, int x, int y, int z,
                                          int64_t cell, uint32_t& mask, uint32_t& lidbits)
{
    if (p.box) return box_classify<Q>(x, y, z, p.nx, p.ny, p.nz, mask, lidbits);
    const uint32_t f = __ldg(flags + cell);
    const int      cls = flag_class(f);
    mask = flag_mask(f);
    lidbits = 0;
    if (is_zouhe_class(cls)) {
        // Zou-He nodes lie on the box faces: moving-wall sources are looked
        // up inside the box only (an out-of-box source is a resting wall)
        const int64_t sy = p.nx, sz = int64_t(p.nx) * p.ny;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            if (!(mask & (1u << q))) continue;
            const int sx = x - Lattice<Q>::cx(q), syy = y - Lattice<Q>::cy(q), szz = z - Lattice<Q>::cz(q);
            if (sx < 0 || syy < 0 || szz < 0 || sx >= p.nx || syy >= p.ny || szz >= p.nz) continue;
            if (source_class(flags, sx + sy * syy + sz * szz) == NGB_CELL_MOVINGWALL) lidbits |= 1u << q;
        }
        return cls;
    }
    if (cls == NGB_CELL_BULK) {
        // A bulk cell on the domain face has sources outside the domain: it is
        // not updated (keeps every access inside the arrays).
        if (x == 0 || y == 0 || z == 0 || x == p.nx - 1 || y == p.ny - 1 || z == p.nz - 1) return NGB_CELL_UNDEFINED;
        if (mask) {
            const int64_t sy = p.nx, sz = int64_t(p.nx) * p.ny;
#pragma unroll
            for (int q = 0; q < Q; q++) {
                if (mask & (1u << q)) {
                    const int64_t src = cell - Lattice<Q>::cx(q) - Lattice<Q>::cy(q) * sy - Lattice<Q>::cz(q) * sz;
                    if (source_class(flags, src) == NGB_CELL_MOVINGWALL) lidbits |= 1u << q;
                }
            }
        }
    }
    return cls;
}

// Outlet node: zero-gradient outflow, copies the x-1 neighbour's populations
// when that neighbour exists (inside the box and not "undefined").
template <int Q, typename S>
__device__ __forceinline__ void outlet_copy(const S* __restrict__ fin, S* __restrict__ fout, int64_t stride, int64_t cell, int x,
                                            const uint32_t* __restrict__ flags)
{
    if (x == 0 || flag_class(__ldg(flags + cell - 1)) == NGB_CELL_UNDEFINED) return;
#pragma unroll
    for (int q = 0; q < Q; q++) fout[q * stride + cell] = fin[q * stride + cell - 1];
}

// ------------------------------------------------------------------ FP64 compute (reference arithmetic)
// D3Q19: the expression shapes of LbmTools.h:78-282 in double (compile with
// --fmad=false for IEEE operation order). D3Q27: the project's per-direction
// BGK (rho = sum f, u = sum c f / rho, eq = rho w (1 + 3cu + 4.5cu^2 - usqr)).
// FP64 BGK of the reference (D3Q19: LbmTools.h:171-282 expression shapes;
// D3Q27: the project's per-direction form), on pulled populations.
template <int Q, typename S>
__device__ __forceinline__ void bgk_f64_ref(const S (&pop)[Q], double omega_, S (&out)[Q])
{
    using L = Lattice<Q>;
    using Cd = double;
    const Cd omega = omega_;
    if constexpr (Q == 19) {
#define P(I) static_cast<Cd>(pop[I])
        const Cd X_M1 = P(0) + P(3) + P(4) + P(5) + P(6);
        const Cd X_P1 = P(10) + P(13) + P(14) + P(15) + P(16);
        const Cd X_0 = P(9) + P(1) + P(2) + P(7) + P(8) + P(11) + P(12) + P(17) + P(18);
        const Cd Y_M1 = P(1) + P(3) + P(7) + P(8) + P(14);
        const Cd Y_P1 = P(4) + P(11) + P(13) + P(17) + P(18);
        const Cd Z_M1 = P(2) + P(5) + P(7) + P(16) + P(18);
        const Cd Z_P1 = P(6) + P(8) + P(12) + P(15) + P(17);
        const Cd rho = X_M1 + X_P1 + X_0;
        const Cd u0 = (X_P1 - X_M1) / rho;
        const Cd u1 = (Y_P1 - Y_M1) / rho;
        const Cd u2 = (Z_P1 - Z_M1) / rho;
        const Cd usqr = 1.5 * (u0 * u0 + u1 * u1 + u2 * u2);
        const Cd cu[9] = {u0, u1, u2, u0 + u1, u0 - u1, u0 + u2, u0 - u2, u1 + u2, u1 - u2};
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const Cd wk = k < 3 ? (1. / 18.) : (1. / 36.);
            const Cd eq = rho * wk * (1. - 3. * cu[k] + 4.5 * cu[k] * cu[k] - usqr);
            const Cd eqopp = eq + rho * wk * 6. * cu[k];
            out[k] = static_cast<S>((1. - omega) * P(k) + omega * eq);
            out[k + 10] = static_cast<S>((1. - omega) * P(k + 10) + omega * eqopp);
        }
        const Cd eq9 = rho * (1. / 3.) * (1. - usqr);
        out[9] = static_cast<S>((1. - omega) * P(9) + omega * eq9);
#undef P
    } else {
        Cd f[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) f[q] = Cd(pop[q]);
        Cd rho = 0, mx = 0, my = 0, mz = 0;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            rho += f[q];
            mx += Cd(L::cx(q)) * f[q];
            my += Cd(L::cy(q)) * f[q];
            mz += Cd(L::cz(q)) * f[q];
        }
        const Cd ux = mx / rho, uy = my / rho, uz = mz / rho;
        const Cd usqr = Cd(1.5) * (ux * ux + uy * uy + uz * uz);
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const Cd cu = Cd(L::cx(q)) * ux + Cd(L::cy(q)) * uy + Cd(L::cz(q)) * uz;
            const Cd eq = rho * Cd(L::w(q)) * (Cd(1) + Cd(3) * cu + Cd(4.5) * cu * cu - usqr);
            out[q] = static_cast<S>((Cd(1) - omega) * f[q] + omega * eq);
        }
    }
}

// Zou-He node (D3Q19) in the reference's FP64 arithmetic: the pull of the
// known populations (wall rule for masked directions), M and K, the boundary
// rho and u, the equilibria of collideBgkUnrolled's shapes (LbmTools.h:198-282),
// the unknowns f_q = f_opp(q) + eq_q - eq_opp(q), and the BGK relaxation
// towards eq(rho, u).
template <typename S>
__device__ __forceinline__ void zouhe_node_f64(const S* __restrict__ fin, S* __restrict__ fout, int64_t cell, int x, int y,
                                               int z, int cls, uint32_t mask, uint32_t lidbits, const DenseParams<double>& p)
{
    using L = Lattice<19>;
    const int64_t sy = p.nx, sz = int64_t(p.nx) * p.ny, stride = p.stride;
    int           a, s;
    zouhe_normal(x, y, z, p.nx, p.ny, p.nz, a, s);
    double pop[19];
#pragma unroll
    for (int q = 0; q < 19; q++) {
        pop[q] = 0.0;
        if (lattice_c<19>(q, a) * s == 1) continue;  // unknown: arrives from outside the box
        if (mask & (1u << q)) {
            const int o = L::opp(q);
            pop[q] = double(__ldg(fin + o * stride + cell)) + ((lidbits & (1u << q)) ? p.wall[1][o] : p.wall[0][o]);
        } else {
            pop[q] = double(__ldg(fin + q * stride + cell - L::cx(q) - L::cy(q) * sy - L::cz(q) * sz));
        }
    }
    double M = 0.0, K = 0.0;
#pragma unroll
    for (int q = 0; q < 19; q++) {
        const int ca = lattice_c<19>(q, a);
        if (ca == 0) M = M + pop[q];
        else if (ca * s == -1) K = K + pop[q];
    }
    double rho, u[3] = {0.0, 0.0, 0.0};
    if (cls == NGB_CELL_PRESSURE) {
        rho = p.zh_rho;
        u[a] = double(s) * (1.0 - (M + 2.0 * K) / rho);
    } else {
        for (int d = 0; d < 3; d++) u[d] = p.zh_u[d];
        rho = (M + 2.0 * K) / (1.0 - double(s) * u[a]);
    }
    const double usqr = 1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    const double cu[9] = {u[0], u[1], u[2], u[0] + u[1], u[0] - u[1], u[0] + u[2], u[0] - u[2], u[1] + u[2], u[1] - u[2]};
    double       eq[19];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const double wk = k < 3 ? (1. / 18.) : (1. / 36.);
        eq[k] = rho * wk * (1. - 3. * cu[k] + 4.5 * cu[k] * cu[k] - usqr);
        eq[k + 10] = eq[k] + rho * wk * 6. * cu[k];
    }
    eq[9] = rho * (1. / 3.) * (1. - usqr);
#pragma unroll
    for (int q = 0; q < 19; q++)
        if (lattice_c<19>(q, a) * s == 1) pop[q] = pop[L::opp(q)] + eq[q] - eq[L::opp(q)];
#pragma unroll
    for (int q = 0; q < 19; q++) fout[q * stride + cell] = S((1. - p.omega) * pop[q] + p.omega * eq[q]);
}

template <int Q, typename S>
__global__ void __launch_bounds__(kLbmBlockX) lbm_dense_f64_kernel(const S* __restrict__ fin, S* __restrict__ fout,
                                                                   const uint32_t* __restrict__ flags, DenseParams<double> p)
{
    using L = Lattice<Q>;
    const int x = blockIdx.x * kLbmBlockX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= p.nx) return;
    const int64_t sy = p.nx, sz = int64_t(p.nx) * p.ny, stride = p.stride;
    const int64_t cell = x + sy * y + sz * z;
    uint32_t      mask, lidbits;
    const int     cls = cell_setup<Q>(p, flags, x, y, z, cell, mask, lidbits);
    if (cls == NGB_CELL_OUTLET) {
        outlet_copy<Q>(fin, fout, stride, cell, x, flags);
        return;
    }
    if (is_zouhe_class(cls)) {
        if constexpr (Q == 19) zouhe_node_f64<S>(fin, fout, cell, x, y, z, cls, mask, lidbits, p);
        return;
    }
    if (cls != NGB_CELL_BULK) return;

    S pop[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) {
        if (mask & (1u << q)) {
            const int o = L::opp(q);
            const S   wt = S((lidbits & (1u << q)) ? p.wall[1][o] : p.wall[0][o]);
            pop[q] = __ldg(fin + o * stride + cell) + wt;
        } else {
            const int64_t src = cell - L::cx(q) - L::cy(q) * sy - L::cz(q) * sz;
            pop[q] = __ldg(fin + q * stride + src);
        }
    }
    S out[Q];
    bgk_f64_ref<Q, S>(pop, p.omega, out);
#pragma unroll
    for (int q = 0; q < Q; q++) fout[q * stride + cell] = out[q];
}

// Whether the FP32-compute launcher runs the analytic cavity as the core + shell kernel pair.
inline bool lbm_dense_split(int Q, int storage, const DenseParams<float>& p)
{
    // D3Q27 with 16-bit storage splits where its core runs as the x-pair kernel (even rows and planes)
    return p.box && p.nx >= 4 && p.ny >= 6 && p.nz >= 6 &&
           (Q == 19 || storage == NGB_STORE_F32 || (p.nx % 2 == 0 && p.stride % 2 == 0));
}

// Host-side launchers (lbm_dense.cu / lbm_dense_f64.cu).
int launch_lbm_dense_f32(int Q, int storage, const void* fin, void* fout, const uint32_t* flags, const DenseParams<float>& p,
                         cudaStream_t s);
int launch_lbm_dense_f64(int Q, const void* fin, void* fout, const uint32_t* flags, const DenseParams<double>& p, cudaStream_t s);

}  // namespace ngb
