// ORACLE — test infrastructure only.
//
// CPU restatement of the Neon lid-driven-cavity LBM path, used by the tests,
// by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
// Nothing in the product library links or calls this code.
//
// Follows (paths relative to the Neon repository):
//   benchmarks/lbm-lid-driven-cavity-flow/src/D3Q19.h:23-132      velocity set, opposites, weights
//   benchmarks/lbm-lid-driven-cavity-flow/src/CellType.h:3-35     cell classification
//   benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h:78-168   pull stream with half-way bounce-back
//   benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h:171-195  macroscopic moments
//   benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h:198-282  unrolled BGK collision
//   benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h:284-325  the iteration container (bulk cells only)
//   benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h:327-376  wall-neighbour mask
//   benchmarks/lbm-lid-driven-cavity-flow/src/RunCavityTwoPop.cu:159-242  problem set-up
//   benchmarks/lbm-lid-driven-cavity-flow/src/Config.cpp:105-111  nu / omega
//   apps/lbmMultiRes/lattice.h:14-77                               D3Q27 velocity set and weights
//
// The arithmetic of the D3Q19 step keeps the reference's expression shapes
// (including its double-precision literals), so that instantiating with
// <double,double> or <float,float> reproduces the reference's own rounding
// on a CPU with FP contraction disabled (-ffp-contract=off).
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>
#include <array>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------- lattices
// D3Q19 in Neon's order: 0..8 "go" directions, 9 the rest population,
// 10..18 the opposites of 0..8 (D3Q19.h:23-44, 62-82).
static const int kC19[19][3] = {
    {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1}, {0, -1, -1}, {0, -1, 1},
    {0, 0, 0},
    {1, 0, 0},  {0, 1, 0},  {0, 0, 1},  {1, 1, 0},   {1, -1, 0}, {1, 0, 1},   {1, 0, -1}, {0, 1, 1},   {0, 1, -1}};
static const double kW19[19] = {
    1. / 18., 1. / 18., 1. / 18., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.,
    1. / 3.,
    1. / 18., 1. / 18., 1. / 18., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
inline int opp19(int q) { return q == 9 ? 9 : (q < 9 ? q + 10 : q - 10); }

// D3Q27 in the order of apps/lbmMultiRes/lattice.h:14-42: index = 9*a + 3*b + c
// with digit 0 -> 0, 1 -> -1, 2 -> +1 for (cx, cy, cz); the rest population first.
inline int d27_digit_to_c(int d) { return d == 0 ? 0 : (d == 1 ? -1 : 1); }
inline int c27(int q, int axis)
{
    const int a = q / 9, b = (q / 3) % 3, c = q % 3;
    return d27_digit_to_c(axis == 0 ? a : (axis == 1 ? b : c));
}
inline int opp27(int q)
{
    auto flip = [](int d) { return d == 0 ? 0 : 3 - d; };
    return 9 * flip(q / 9) + 3 * flip((q / 3) % 3) + flip(q % 3);
}
inline double w27(int q)
{
    int nz = (c27(q, 0) != 0) + (c27(q, 1) != 0) + (c27(q, 2) != 0);
    return nz == 0 ? 8. / 27. : (nz == 1 ? 2. / 27. : (nz == 2 ? 1. / 54. : 1. / 216.));
}

// ---------------------------------------------------------------- cell type
// CellType.h:3-35: {uint32 wallNghBitflag; classification}.
// outlet (zero-gradient outflow: copies the x-1 neighbour) is the project's own addition;
// pressure / velocity are Zou-He boundary nodes (the classes of
// benchmarks/lbm-flow-over-sphere/src/CellType.h), defined below.
enum Classification : int { bounceBack = 0, movingWall = 1, bulk = 2, undefined = 3, outlet = 4, pressure = 5, velocity = 6 };
inline bool is_zouhe(int c) { return c == pressure || c == velocity; }
inline bool is_fluid(int c) { return c == bulk || c == outlet || is_zouhe(c); }

// ---------------------------------------------------------------- Zou-He boundary nodes
// The project's definition of the pressure / velocity boundary of the
// flow-over-sphere benchmark (LbmContainers.h:53-290 there), as the
// non-equilibrium bounce-back of Zou & He (1997) on D3Q19:
// * a Zou-He node lies on a face of the box; its inward normal n is that of
//   the first face it lies on, in the order x = 0, x = nx-1, y = 0, y = ny-1,
//   z = 0, z = nz-1 (axis a, sign s = +1 on the low face, -1 on the high one);
// * it is updated every step: the 5 populations with s c_a = +1 arrive from
//   outside the box and are unknown; the others stream (pull, with the wall
//   rule for masked directions; an out-of-box source counts as a resting wall);
// * M = sum of the known populations with c_a = 0, K = sum of those with
//   s c_a = -1 (q ascending); pressure nodes take rho = rho_b and the normal
//   velocity s u_a = 1 - (M + 2K) / rho_b, tangential velocity 0 (as the
//   reference's streamAndZouhe); velocity nodes take u = u_b and
//   rho = (M + 2K) / (1 - s u_b,a);
// * the unknowns follow f_q = f_opp(q) + eq_q - eq_opp(q), and the node
//   collides with eq(rho, u) of the boundary values (the reference collides
//   its Zou-He nodes with the boundary rho and u, not with re-summed moments).
struct ZouHe {
    double rho = 1.0;
    double u[3] = {0.0, 0.0, 0.0};
};
inline void zouhe_normal(int x, int y, int z, int nx, int ny, int nz, int& a, int& s)
{
    if (x == 0) a = 0, s = 1;
    else if (x == nx - 1) a = 0, s = -1;
    else if (y == 0) a = 1, s = 1;
    else if (y == ny - 1) a = 1, s = -1;
    else if (z == 0) a = 2, s = 1;
    else a = 2, s = -1;
}
struct CellType {
    uint32_t wallNghBitflag = 0;
    int      classification = bulk;
};

// ---------------------------------------------------------------- storage conversions
// IEEE-754 binary16 / bfloat16 with round-to-nearest-even, written from the
// format definitions (used for the equilibrium-offset storage forms).
inline uint16_t f32_to_f16(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return uint16_t(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return uint16_t(sign | 0x7c00u);  // rounds to infinity
    if (ax < 0x38800000u) {                                   // half subnormal or zero
        const int e = int(ax >> 23);
        if (e == 0) return uint16_t(sign);
        const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        const int      shift = 126 - e;
        if (shift >= 25) return uint16_t(sign);
        uint32_t       r = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u);
        const uint32_t half = 1u << (shift - 1);
        if (rem > half || (rem == half && (r & 1u))) r++;
        return uint16_t(sign | r);
    }
    uint32_t       r = ((((ax >> 23) - 127u + 15u) << 10) | ((ax & 0x7fffffu) >> 13));
    const uint32_t rem = ax & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
    return uint16_t(sign | r);
}
inline float f16_to_f32(uint16_t h)
{
    const uint32_t sign = uint32_t(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu;
    const uint32_t m = h & 0x3ffu;
    uint32_t       x;
    if (e == 0) {
        if (m == 0) {
            x = sign;
        } else {  // subnormal: m * 2^-24
            float v = float(m) * (1.0f / 16777216.0f);
            std::memcpy(&x, &v, 4);
            x |= sign;
        }
    } else if (e == 31) {
        x = sign | 0x7f800000u | (m << 13);
    } else {
        x = sign | ((e - 15u + 127u) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}
// IEEE binary16 with round toward zero (truncation of the dropped bits).
inline uint16_t f32_to_f16_rz(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return uint16_t(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x47800000u) return uint16_t(sign | 0x7bffu);  // |f| >= 65536: largest finite (toward zero)
    if (ax < 0x38800000u) {                                   // half subnormal or zero
        const int e = int(ax >> 23);
        if (e == 0) return uint16_t(sign);
        const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        const int      shift = 126 - e;
        if (shift >= 32) return uint16_t(sign);
        return uint16_t(sign | (m >> shift));
    }
    return uint16_t(sign | ((((ax >> 23) - 127u + 15u) << 10) | ((ax & 0x7fffffu) >> 13)));
}

// Stochastic rounding of FP16 offset storage (the library's F16SR): the random
// bits r of cell i, population q, step seed s,
//   h = mix32(lo32(i >> 1) ^ (hi32(i >> 1) * 0x9E3779B1) ^ (s * 0x85EBCA77))
//   hq = (h ^ (q * 0x9E3779B9)) * 0xC2B2AE35;  r = i odd ? (hq >> 16) & 0x1FFF : hq & 0x1FFF
// (mix32 is Wellons' lowbias32 integer hash) are added, in units of 2^-13 of
// the FP16 result's ulp, to the magnitude of the (scaled) value, which is
// then truncated: the conversion the GPU's cvt.rs.f16x2.f32 performs with
// one random word per pair (bits 0-12 for the low result, 16-28 for the high),
// pinned bit for bit against that instruction's outputs in the tests.
inline uint32_t dither_mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
inline uint32_t dither_bits(uint64_t cell, int q, uint32_t seed)
{
    const uint64_t pr = cell >> 1;
    const uint32_t h = dither_mix32(uint32_t(pr) ^ (uint32_t(pr >> 32) * 0x9E3779B1u) ^ (seed * 0x85EBCA77u));
    const uint32_t hq = (h ^ (uint32_t(q) * 0x9E3779B9u)) * 0xC2B2AE35u;
    return (cell & 1) ? ((hq >> 16) & 0x1fffu) : (hq & 0x1fffu);
}
// r in [0, 8192). Normal FP16 results: the FP32 significand keeps 13 bits
// below the FP16 ulp, so adding r to the FP32 bit pattern (a carry may raise
// the exponent) and truncating is the rule; a sum of 2^16 or more overflows
// to infinity (no saturation). FP16 subnormal results (|f| < 2^-14, ulp
// 2^-24): floor((floor(|f| 2^37) + r) / 2^13) ulps.
inline uint16_t f32_to_f16_sr(float f, uint32_t r)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax < 0x38800000u) {
        const int      e = int(ax >> 23);  // |f| = m 2^(e - 150) for e >= 1
        const int      shift = 113 - e;    // floor(|f| 2^37) = m >> shift
        const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        const uint32_t fx = (e == 0 || shift >= 32) ? 0u : (m >> shift);
        return uint16_t(sign | ((fx + r) >> 13));
    }
    if (ax >= 0x7f800000u) return f32_to_f16_rz(f);  // infinity, NaN
    x += r;                                           // r < 2^13: may carry into the exponent
    if ((x & 0x7fffffffu) >= 0x47800000u) return uint16_t(sign | 0x7c00u);  // rounded to 2^16 or beyond: overflow
    float g;
    std::memcpy(&g, &x, 4);
    return f32_to_f16_rz(g);
}

inline uint16_t f32_to_bf16(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    if ((x & 0x7fffffffu) > 0x7f800000u) return uint16_t((x >> 16) | 0x40u);
    const uint32_t lsb = (x >> 16) & 1u;
    x += 0x7fffu + lsb;
    return uint16_t(x >> 16);
}
inline float bf16_to_f32(uint16_t b)
{
    uint32_t x = uint32_t(b) << 16;
    float    f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ---------------------------------------------------------------- set-up
// Config.cpp:105-111
inline double cavity_omega(int N, double ulb, double Re)
{
    const double nu = ulb * double(N - 2) / Re;
    return 1. / (3. * nu + 0.5);
}

// Stored value of population k at a wall node (RunCavityTwoPop.cu:168-206):
// 0 for resting walls, -6 w_k u_lb (c_k . u_lid) on the moving lid.
inline double wall_term19(int k, bool lid, double ulb)
{
    if (!lid) return 0.0;
    const double ulid[3] = {1., 0., 0.};
    return -6. * kW19[k] * ulb * (kC19[k][0] * ulid[0] + kC19[k][1] * ulid[1] + kC19[k][2] * ulid[2]);
}
inline double wall_term27(int k, bool lid, double ulb)
{
    if (!lid) return 0.0;
    return -6. * w27(k) * ulb * double(c27(k, 0));
}

inline bool on_box_face(int x, int y, int z, int nx, int ny, int nz)
{
    return x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
}

// Population layout of a single-partition Neon dField (dField_imp.h:71-77):
// element (x, y, z, q) at x + y*nx + z*nx*ny + q*nx*ny*nz.
inline size_t lin(int x, int y, int z, int nx, int ny) { return size_t(x) + size_t(nx) * (size_t(y) + size_t(ny) * size_t(z)); }

template <typename S>
void cavity_init_populations(int nx, int ny, int nz, int Q, double ulb, S* pop)
{
    const size_t V = size_t(nx) * ny * nz;
    for (int q = 0; q < Q; q++)
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    double w = Q == 19 ? kW19[q] : w27(q);
                    double val = w;
                    if (on_box_face(x, y, z, nx, ny, nz)) {
                        const bool lid = (y == ny - 1);
                        val = Q == 19 ? wall_term19(q, lid, ulb) : wall_term27(q, lid, ulb);
                    }
                    pop[q * V + lin(x, y, z, nx, ny)] = S(val);
                }
}

inline void cavity_init_flags(int nx, int ny, int nz, CellType* flag)
{
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                CellType c;
                c.classification = bulk;
                if (on_box_face(x, y, z, nx, ny, nz)) c.classification = (y == ny - 1) ? movingWall : bounceBack;
                flag[lin(x, y, z, nx, ny)] = c;
            }
}

// LbmTools.h:327-376: for bulk cells, bit q is set iff the pull source x - c_q
// is not bulk (a missing neighbour counts as "undefined", i.e. not bulk).
inline void compute_wall_mask(int nx, int ny, int nz, int Q, CellType* flag)
{
    std::vector<CellType> in(flag, flag + size_t(nx) * ny * nz);
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                CellType c = in[lin(x, y, z, nx, ny)];
                c.wallNghBitflag = 0;
                if (c.classification != bulk && !is_zouhe(c.classification)) continue;
                for (int q = 0; q < Q; q++) {
                    const int cx = Q == 19 ? kC19[q][0] : c27(q, 0);
                    const int cy = Q == 19 ? kC19[q][1] : c27(q, 1);
                    const int cz = Q == 19 ? kC19[q][2] : c27(q, 2);
                    if (cx == 0 && cy == 0 && cz == 0) continue;
                    const int sx = x - cx, sy = y - cy, sz = z - cz;
                    int       cls = undefined;
                    if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) cls = in[lin(sx, sy, sz, nx, ny)].classification;
                    if (!is_fluid(cls)) c.wallNghBitflag |= (uint32_t(1) << q);
                }
                flag[lin(x, y, z, nx, ny)] = c;
            }
}

// ---------------------------------------------------------------- D3Q19 step (reference arithmetic)
// One pull stream-collide step over every bulk cell (LbmTools.h:284-325).
// S = storage type, C = compute type.
// Reference-shape equilibria of D3Q19 (collideBgkUnrolled, LbmTools.h:198-282):
// eq[k] for the go directions k = 0..8, eq[k+10] = eq[k] + rho w 6 (c_{k+10}.u), eq[9].
template <typename C>
void d3q19_eq(C rho, C u0, C u1, C u2, C usqr, C* eq)
{
    const C cu[9] = {u0, u1, u2, u0 + u1, u0 - u1, u0 + u2, u0 - u2, u1 + u2, u1 - u2};
    for (int k = 0; k < 9; k++) {
        const double wk = k < 3 ? (1. / 18.) : (1. / 36.);
        eq[k] = rho * wk * (1. - 3. * cu[k] + 4.5 * cu[k] * cu[k] - usqr);
        eq[k + 10] = eq[k] + rho * wk * 6. * cu[k];
    }
    eq[9] = rho * (1. / 3.) * (1. - usqr);
}

// Zou-He node in the reference's arithmetic (FP64 / FP32 compute C).
// `wall` gives the wall term of a masked direction by the source's class.
template <typename S, typename C, typename At, typename WallTerm>
void zouhe_node_ref(int x, int y, int z, int nx, int ny, int nz, const CellType& cell, C omega, const ZouHe& zh, At at,
                    WallTerm wall, C* out)
{
    int a, s;
    zouhe_normal(x, y, z, nx, ny, nz, a, s);
    C pop[19];
    for (int q = 0; q < 19; q++) {
        if (kC19[q][a] * s == 1) continue;  // unknown
        const int sx = x - kC19[q][0], sy = y - kC19[q][1], sz = z - kC19[q][2];
        if (cell.wallNghBitflag & (uint32_t(1) << q)) {
            const bool inside = sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz;
            pop[q] = static_cast<C>(at(x, y, z, opp19(q))) + C(wall(inside, sx, sy, sz, opp19(q)));
        } else {
            pop[q] = static_cast<C>(at(sx, sy, sz, q));
        }
    }
    C M = 0, K = 0;
    for (int q = 0; q < 19; q++) {
        if (kC19[q][a] == 0) M = M + pop[q];
        else if (kC19[q][a] * s == -1) K = K + pop[q];
    }
    C rho, u[3] = {0, 0, 0};
    if (cell.classification == pressure) {
        rho = C(zh.rho);
        u[a] = C(s) * (C(1) - (M + C(2) * K) / rho);
    } else {
        for (int d = 0; d < 3; d++) u[d] = C(zh.u[d]);
        rho = (M + C(2) * K) / (C(1) - C(s) * u[a]);
    }
    const C usqr = 1.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    C       eq[19];
    d3q19_eq<C>(rho, u[0], u[1], u[2], usqr, eq);
    for (int q = 0; q < 19; q++)
        if (kC19[q][a] * s == 1) pop[q] = pop[opp19(q)] + eq[q] - eq[opp19(q)];
    for (int q = 0; q < 19; q++) out[q] = (1. - omega) * pop[q] + omega * eq[q];
}

template <typename S, typename C>
void d3q19_step(int nx, int ny, int nz, const S* fin, S* fout, const CellType* flag, C omega,
                int z_begin = 0, int z_end = -1, const ZouHe* zh = nullptr, const double (*wallt)[27] = nullptr)
{
    const size_t V = size_t(nx) * ny * nz;
    if (z_end < 0) z_end = nz;
    auto at = [&](int x, int y, int z, int q) -> S { return fin[size_t(q) * V + lin(x, y, z, nx, ny)]; };
    auto zwall = [&](bool inside, int sx, int sy, int sz, int q) -> double {
        if (!wallt) return 0.0;
        if (!inside) return wallt[0][q];  // out of the box: a resting wall
        return flag[lin(sx, sy, sz, nx, ny)].classification == movingWall ? wallt[1][q] : wallt[0][q];
    };
    for (int z = z_begin; z < z_end; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const CellType cell = flag[lin(x, y, z, nx, ny)];
                if (is_zouhe(cell.classification)) {
                    if (!zh) continue;
                    C out[19];
                    zouhe_node_ref<S, C>(x, y, z, nx, ny, nz, cell, omega, *zh, at, zwall, out);
                    for (int q = 0; q < 19; q++) fout[size_t(q) * V + lin(x, y, z, nx, ny)] = static_cast<S>(out[q]);
                    continue;
                }
                if (cell.classification == outlet) {
                    if (x > 0 && flag[lin(x - 1, y, z, nx, ny)].classification != undefined)
                        for (int q = 0; q < 19; q++) fout[size_t(q) * V + lin(x, y, z, nx, ny)] = at(x - 1, y, z, q);
                    continue;
                }
                if (cell.classification != bulk) continue;
                const uint32_t m = cell.wallNghBitflag;
                S              pop[19];
                // Pull stream (LbmTools.h:78-168): population q arrives from x - c_q;
                // if that node is a wall, the opposite population of this cell is
                // reflected and the wall's stored term is added.
                for (int go = 0; go < 9; go++) {
                    const int bk = go + 10;
                    const int gx = kC19[go][0], gy = kC19[go][1], gz = kC19[go][2];
                    if (m & (uint32_t(1) << go))
                        pop[go] = at(x, y, z, bk) + at(x - gx, y - gy, z - gz, bk);
                    else
                        pop[go] = at(x - gx, y - gy, z - gz, go);
                    if (m & (uint32_t(1) << bk))
                        pop[bk] = at(x, y, z, go) + at(x + gx, y + gy, z + gz, go);
                    else
                        pop[bk] = at(x + gx, y + gy, z + gz, bk);
                }
                pop[9] = at(x, y, z, 9);

                // Macroscopic moments (LbmTools.h:171-195), grouped sums in the same order.
#define P(I) static_cast<C>(pop[I])
                const C X_M1 = P(0) + P(3) + P(4) + P(5) + P(6);
                const C X_P1 = P(10) + P(13) + P(14) + P(15) + P(16);
                const C X_0 = P(9) + P(1) + P(2) + P(7) + P(8) + P(11) + P(12) + P(17) + P(18);
                const C Y_M1 = P(1) + P(3) + P(7) + P(8) + P(14);
                const C Y_P1 = P(4) + P(11) + P(13) + P(17) + P(18);
                const C Z_M1 = P(2) + P(5) + P(7) + P(16) + P(18);
                const C Z_P1 = P(6) + P(8) + P(12) + P(15) + P(17);
                const C rho = X_M1 + X_P1 + X_0;
                const C u0 = (X_P1 - X_M1) / rho;
                const C u1 = (Y_P1 - Y_M1) / rho;
                const C u2 = (Z_P1 - Z_M1) / rho;
                const C usqr = 1.5 * (u0 * u0 + u1 * u1 + u2 * u2);

                // BGK (LbmTools.h:198-282): the "go" equilibria, their opposites via
                // + rho w 6 (c.u), then (1 - omega) f + omega eq.
                const C cu[9] = {u0, u1, u2, u0 + u1, u0 - u1, u0 + u2, u0 - u2, u1 + u2, u1 - u2};
                for (int k = 0; k < 9; k++) {
                    const double wk = k < 3 ? (1. / 18.) : (1. / 36.);
                    // cu[k] here is c_{opp k} . u; the go direction has c_k . u = -cu[k].
                    const C eq = rho * wk * (1. - 3. * cu[k] + 4.5 * cu[k] * cu[k] - usqr);
                    const C eqopp = eq + rho * wk * 6. * cu[k];
                    const C out = (1. - omega) * P(k) + omega * eq;
                    const C outopp = (1. - omega) * P(k + 10) + omega * eqopp;
                    fout[size_t(k) * V + lin(x, y, z, nx, ny)] = static_cast<S>(out);
                    fout[size_t(k + 10) * V + lin(x, y, z, nx, ny)] = static_cast<S>(outopp);
                }
                {
                    const C eq9 = rho * (1. / 3.) * (1. - usqr);
                    const C out9 = (1. - omega) * P(9) + omega * eq9;
                    fout[size_t(9) * V + lin(x, y, z, nx, ny)] = static_cast<S>(out9);
                }
#undef P
            }
}

// ---------------------------------------------------------------- generic BGK step (D3Q19 / D3Q27, any storage)
// The project's own D3Q19/D3Q27 BGK in a plain per-direction form, used for
// D3Q27 (which the reference does not have as single-resolution BGK) and for
// the equilibrium-offset storage forms. Storage is accessed through Load/Store
// functors so that f16/bf16 offsets (g = f - w) share this code.
//   rho = sum_q f_q; u = sum_q c_q f_q / rho
//   eq_q = rho w_q (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 |u|^2)
//   f_q' = (1 - omega) f_q + omega eq_q
// Wall rule identical to the D3Q19 reference step: bit q set -> f(x, opp q) + wall term.
template <typename C, int Q, typename Load, typename Store, typename WallTerm>
void bgk_step_generic(int nx, int ny, int nz, const CellType* flag, C omega, Load load, Store store, WallTerm wall,
                      int z_begin = 0, int z_end = -1)
{
    if (z_end < 0) z_end = nz;
    int    cx[Q], cy[Q], cz[Q], op[Q];
    double w[Q];
    for (int q = 0; q < Q; q++) {
        cx[q] = Q == 19 ? kC19[q][0] : c27(q, 0);
        cy[q] = Q == 19 ? kC19[q][1] : c27(q, 1);
        cz[q] = Q == 19 ? kC19[q][2] : c27(q, 2);
        op[q] = Q == 19 ? opp19(q) : opp27(q);
        w[q] = Q == 19 ? kW19[q] : w27(q);
    }
    for (int z = z_begin; z < z_end; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const CellType cell = flag[lin(x, y, z, nx, ny)];
                if (cell.classification == outlet) {
                    if (x > 0 && flag[lin(x - 1, y, z, nx, ny)].classification != undefined)
                        for (int q = 0; q < Q; q++) store(x, y, z, q, load(x - 1, y, z, q));
                    continue;
                }
                if (cell.classification != bulk) continue;
                C f[Q];
                for (int q = 0; q < Q; q++) {
                    const int sx = x - cx[q], sy = y - cy[q], sz = z - cz[q];
                    if (cell.wallNghBitflag & (uint32_t(1) << q)) {
                        int cls = undefined;
                        if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) cls = flag[lin(sx, sy, sz, nx, ny)].classification;
                        f[q] = load(x, y, z, op[q]) + wall(cls, op[q]);
                    } else {
                        f[q] = load(sx, sy, sz, q);
                    }
                }
                C rho = 0, mx = 0, my = 0, mz = 0;
                for (int q = 0; q < Q; q++) {
                    rho += f[q];
                    mx += C(cx[q]) * f[q];
                    my += C(cy[q]) * f[q];
                    mz += C(cz[q]) * f[q];
                }
                const C ux = mx / rho, uy = my / rho, uz = mz / rho;
                const C usqr = C(1.5) * (ux * ux + uy * uy + uz * uz);
                for (int q = 0; q < Q; q++) {
                    const C cu = C(cx[q]) * ux + C(cy[q]) * uy + C(cz[q]) * uz;
                    const C eq = rho * C(w[q]) * (C(1) + C(3) * cu + C(4.5) * cu * cu - usqr);
                    const C out = (C(1) - omega) * f[q] + omega * eq;
                    store(x, y, z, q, out);
                }
            }
}

// ---------------------------------------------------------------- shifted FP32 BGK
// The project's equilibrium-shifted FP32 form (used for FP32 storage and for
// the FP16/BF16 offset storage; no reference counterpart). Storage holds
// f_q (FP32) or g_q = f_q - w_q (16-bit). Every operation is IEEE single
// precision in this exact order, fused multiply-adds written as std::fmaf:
//   drho = g_0 + g_1 + ... + g_{Q-1};  j_a = (sum_{c_a>0} g) - (sum_{c_a<0} g), q ascending
//   rho = 1 + drho; inv = 1 / rho; u_a = j_a * inv
//   usq = fma(uz, uz, fma(uy, uy, ux * ux)); rus = rho * (1.5 * usq); base = drho - rus
//   u3_a = 3 * u_a; per weight w: wr = w * rho, wb = w * base
//   per q: t = c_q . u3 (signed adds in x, y, z order); a = fma(0.5 * t, t, t)
//          eqg = fma(wr, a, wb); g' = fma(omega, eqg - g, g)
// Wall rule as the reference step: bit q set -> g(x, opp q) + wall term.
// Zou-He node in the shifted FP32 form (see ZouHe above), g = f - w:
//   M, K as above on g (float adds, q ascending), mk = M + (K + K);
//   pressure: drho = float(rho_b - 1), rho = 1 + drho, s u_a = (drho - mk) / rho;
//   velocity: u = float(u_b), un = s u_a, drho = (mk + un) / (1 - un), rho = 1 + drho;
//   unknowns: g_q = fma((2 w_q) rho, t_q, g_opp(q)) with t_q = c_q . 3u
//   (f_q - f_opp(q) = eq_q - eq_opp(q) = 6 w rho c_q.u); then the relaxation
//   of the shifted BGK with these drho and u.
template <int Q>
void zouhe_node_shifted(int x, int y, int z, int nx, int ny, int nz, const CellType& cell, float omega, float zh_drho,
                        const float* zh_u, const float* g_known, float* out)
{
    int a, s;
    zouhe_normal(x, y, z, nx, ny, nz, a, s);
    float g[19];
    for (int q = 0; q < 19; q++) g[q] = g_known[q];
    float M = 0.f, K = 0.f;
    for (int q = 0; q < 19; q++) {
        if (kC19[q][a] == 0) M = M + g[q];
        else if (kC19[q][a] * s == -1) K = K + g[q];
    }
    const float mk = M + (K + K);
    float       u[3] = {0.f, 0.f, 0.f}, drho, rho;
    if (cell.classification == pressure) {
        drho = zh_drho;
        rho = 1.f + drho;
        u[a] = float(s) * ((drho - mk) / rho);
    } else {
        for (int d = 0; d < 3; d++) u[d] = zh_u[d];
        const float un = float(s) * u[a];
        drho = (mk + un) / (1.f - un);
        rho = 1.f + drho;
    }
    const float u3[3] = {3.f * u[0], 3.f * u[1], 3.f * u[2]};
    auto        tdot = [&](int q) {
        float t = 0.f;
        bool  started = false;
        for (int d = 0; d < 3; d++) {
            if (kC19[q][d] == 0) continue;
            if (!started) {
                t = kC19[q][d] > 0 ? u3[d] : -u3[d];
                started = true;
            } else {
                t = kC19[q][d] > 0 ? t + u3[d] : t - u3[d];
            }
        }
        return t;
    };
    for (int q = 0; q < 19; q++)
        if (kC19[q][a] * s == 1) g[q] = std::fmaf((2.f * float(kW19[q])) * rho, tdot(q), g[opp19(q)]);
    const float usq = std::fmaf(u[2], u[2], std::fmaf(u[1], u[1], u[0] * u[0]));
    const float rus = rho * (1.5f * usq);
    const float base = drho - rus;
    for (int q = 0; q < 19; q++) {
        const float w = float(kW19[q]), wr = w * rho, wb = w * base;
        const float t = tdot(q);
        const float aa = std::fmaf(0.5f * t, t, t);
        const float eqg = std::fmaf(wr, aa, wb);
        out[q] = std::fmaf(omega, eqg - g[q], g[q]);
    }
}

template <int Q, typename LoadG, typename StoreG, typename WallTerm>
void bgk_step_shifted(int nx, int ny, int nz, const CellType* flag, float omega, LoadG loadg, StoreG storeg, WallTerm wall,
                      int z_begin = 0, int z_end = -1, const ZouHe* zh = nullptr)
{
    if (z_end < 0) z_end = nz;
    int   c[Q][3], op[Q];
    float w[Q];
    for (int q = 0; q < Q; q++) {
        for (int a = 0; a < 3; a++) c[q][a] = Q == 19 ? kC19[q][a] : c27(q, a);
        op[q] = Q == 19 ? opp19(q) : opp27(q);
        w[q] = float(Q == 19 ? kW19[q] : w27(q));
    }
    for (int z = z_begin; z < z_end; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const CellType cell = flag[lin(x, y, z, nx, ny)];
                if (cell.classification == outlet) {
                    if (x > 0 && flag[lin(x - 1, y, z, nx, ny)].classification != undefined)
                        for (int q = 0; q < Q; q++) storeg(x, y, z, q, loadg(x - 1, y, z, q));
                    continue;
                }
                if (Q == 19 && is_zouhe(cell.classification)) {
                    if (!zh) continue;
                    int za, zs;
                    zouhe_normal(x, y, z, nx, ny, nz, za, zs);
                    float gk[19] = {}, zo[19];
                    for (int q = 0; q < 19; q++) {
                        if (c[q][za] * zs == 1) continue;
                        const int sx = x - c[q][0], sy = y - c[q][1], sz = z - c[q][2];
                        if (cell.wallNghBitflag & (uint32_t(1) << q)) {
                            int cls = undefined;
                            if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) cls = flag[lin(sx, sy, sz, nx, ny)].classification;
                            gk[q] = loadg(x, y, z, op[q]) + float(wall(cls, op[q]));
                        } else {
                            gk[q] = loadg(sx, sy, sz, q);
                        }
                    }
                    const float zu[3] = {float(zh->u[0]), float(zh->u[1]), float(zh->u[2])};
                    zouhe_node_shifted<19>(x, y, z, nx, ny, nz, cell, omega, float(zh->rho - 1.0), zu, gk, zo);
                    for (int q = 0; q < 19; q++) storeg(x, y, z, q, zo[q]);
                    continue;
                }
                if (cell.classification != bulk) continue;
                float g[Q];
                for (int q = 0; q < Q; q++) {
                    const int sx = x - c[q][0], sy = y - c[q][1], sz = z - c[q][2];
                    if (cell.wallNghBitflag & (uint32_t(1) << q)) {
                        int cls = undefined;
                        if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) cls = flag[lin(sx, sy, sz, nx, ny)].classification;
                        g[q] = loadg(x, y, z, op[q]) + float(wall(cls, op[q]));
                    } else {
                        g[q] = loadg(sx, sy, sz, q);
                    }
                }
                float drho = g[0];
                for (int q = 1; q < Q; q++) drho = drho + g[q];
                float jp[3] = {0, 0, 0}, jm[3] = {0, 0, 0};
                bool  sp[3] = {false, false, false}, sm[3] = {false, false, false};
                for (int q = 0; q < Q; q++)
                    for (int a = 0; a < 3; a++) {
                        if (c[q][a] > 0) {
                            jp[a] = sp[a] ? jp[a] + g[q] : g[q];
                            sp[a] = true;
                        } else if (c[q][a] < 0) {
                            jm[a] = sm[a] ? jm[a] + g[q] : g[q];
                            sm[a] = true;
                        }
                    }
                const float jx = jp[0] - jm[0], jy = jp[1] - jm[1], jz = jp[2] - jm[2];
                const float rho = 1.f + drho;
                const float inv = 1.f / rho;
                const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
                const float usq = std::fmaf(uz, uz, std::fmaf(uy, uy, ux * ux));
                const float rus = rho * (1.5f * usq);
                const float base = drho - rus;
                const float u3[3] = {3.f * ux, 3.f * uy, 3.f * uz};
                for (int q = 0; q < Q; q++) {
                    const float wr = w[q] * rho, wb = w[q] * base;
                    float       t = 0.f;
                    bool        started = false;
                    for (int a = 0; a < 3; a++) {
                        if (c[q][a] == 0) continue;
                        if (!started) {
                            t = c[q][a] > 0 ? u3[a] : -u3[a];
                            started = true;
                        } else {
                            t = c[q][a] > 0 ? t + u3[a] : t - u3[a];
                        }
                    }
                    const float a = std::fmaf(0.5f * t, t, t);
                    const float eqg = std::fmaf(wr, a, wb);
                    storeg(x, y, z, q, std::fmaf(omega, eqg - g[q], g[q]));
                }
            }
}

// Density and velocity (LbmTools.h:383-437, computeRhoAndU), in double:
// bulk cells pull their populations exactly like the step (wall rule
// included) and take rho = sum f, u = sum c f / rho; moving-wall cells report
// rho = 1 and u_a = f_a / (6/18) from their stored lid term (a = 0, 1, 2 in
// the D3Q19 order; D3Q27 moving walls report 0); every other cell 0.
template <typename Load, typename WallTerm>
void rho_u_field(int nx, int ny, int nz, int Q, const CellType* flag, Load load, WallTerm wall, double* rho_out,
                 double* u /* 3*V, SoA */)
{
    const size_t V = size_t(nx) * ny * nz;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const size_t i = lin(x, y, z, nx, ny);
                double       rho = 0, m[3] = {0, 0, 0};
                if (flag[i].classification == bulk) {
                    for (int q = 0; q < Q; q++) {
                        const int cx = Q == 19 ? kC19[q][0] : c27(q, 0);
                        const int cy = Q == 19 ? kC19[q][1] : c27(q, 1);
                        const int cz = Q == 19 ? kC19[q][2] : c27(q, 2);
                        const int o = Q == 19 ? opp19(q) : opp27(q);
                        double    f;
                        if (flag[i].wallNghBitflag & (uint32_t(1) << q)) {
                            const int sx = x - cx, sy = y - cy, sz = z - cz;
                            int       cls = undefined;
                            if (sx >= 0 && sy >= 0 && sz >= 0 && sx < nx && sy < ny && sz < nz) cls = flag[lin(sx, sy, sz, nx, ny)].classification;
                            f = load(x, y, z, o) + wall(cls, o);
                        } else {
                            f = load(x - cx, y - cy, z - cz, q);
                        }
                        rho += f;
                        m[0] += double(cx) * f, m[1] += double(cy) * f, m[2] += double(cz) * f;
                    }
                    for (int a = 0; a < 3; a++) m[a] /= rho;
                } else if (flag[i].classification == movingWall) {
                    rho = 1.0;
                    for (int a = 0; a < 3; a++) m[a] = Q == 19 ? wall(movingWall, a) / (6. * 1. / 18.) : 0.0;
                }
                if (rho_out) rho_out[i] = rho;
                for (int a = 0; a < 3; a++) u[a * V + i] = m[a];
            }
}

}  // namespace oracle
