// ORACLE — test infrastructure only.
//
// C-ABI entry points over the CPU restatements in lbm_oracle.hpp,
// bgrid_oracle.hpp and poisson_oracle.hpp. Loaded with ctypes by the tests,
// by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as
// the checker or the timed CPU baseline, never as the product path.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -shared -fPIC
// (FP contraction off so that FP64 results are the IEEE operation order).
#include <cstdint>
#include <cstring>
#include <vector>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lbm_oracle.hpp"
#include "bgrid_oracle.hpp"
#include "poisson_oracle.hpp"

using namespace oracle;

namespace {

enum Storage { ST_F64 = 0, ST_F32 = 1, ST_F16OFF = 2, ST_BF16OFF = 3, ST_F16SR = 4 };
// FP16 offset storage holds fp16(2^14 g) (the library's NGB_F16OFF_SCALE); both factors are exact
constexpr float kF16Up = 16384.0f, kF16Down = 1.0f / 16384.0f;
enum ComputeMode { CM_REFERENCE = 0, CM_GENERIC = 1, CM_SHIFTED = 2 };

// Flags are exchanged with the tests in the packed form used by the GPU
// library: bits 0..26 wall-neighbour mask, bits 28..31 classification.
inline CellType unpack(uint32_t f)
{
    CellType c;
    c.wallNghBitflag = f & 0x07ffffffu;
    c.classification = int(f >> 28);
    return c;
}
inline uint32_t pack(const CellType& c) { return (c.wallNghBitflag & 0x07ffffffu) | (uint32_t(c.classification) << 28); }

double   g_wall[4][27];  // wall terms by classification (set per run)
uint32_t g_dither_seed = 0;  // F16SR: step t of a run uses seed g_dither_seed + (t mod 32)
ZouHe  g_zh;           // Zou-He boundary values (orc_set_zouhe)

double weight(int Q, int q) { return Q == 19 ? kW19[q] : w27(q); }

template <typename C, int Q, typename S, typename ToC, typename FromC>
void generic_run(int nx, int ny, int nz, const CellType* flag, double omega, S* a, S* b, int steps, ToC toC, FromC fromC, int threads)
{
    const size_t V = size_t(nx) * ny * nz;
    for (int t = 0; t < steps; t++) {
        const S* fin = (t % 2 == 0) ? a : b;
        S*       fout = (t % 2 == 0) ? b : a;
        auto     load = [&](int x, int y, int z, int q) -> C { return toC(fin[size_t(q) * V + lin(x, y, z, nx, ny)], q); };
        auto     store = [&](int x, int y, int z, int q, C v) { fout[size_t(q) * V + lin(x, y, z, nx, ny)] = fromC(v, q); };
        auto     wall = [&](int cls, int q) -> C { return C(cls == movingWall ? g_wall[1][q] : g_wall[0][q]); };
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int z = 0; z < nz; z++) bgk_step_generic<C, Q>(nx, ny, nz, flag, C(omega), load, store, wall, z, z + 1);
    }
}

template <int Q, typename S, typename ToG, typename FromG>
void shifted_run(int nx, int ny, int nz, const CellType* flag, float omega, S* a, S* b, int steps, ToG toG, FromG fromG, int threads)
{
    const size_t V = size_t(nx) * ny * nz;
    for (int t = 0; t < steps; t++) {
        const S* fin = (t % 2 == 0) ? a : b;
        S*       fout = (t % 2 == 0) ? b : a;
        auto     loadg = [&](int x, int y, int z, int q) -> float { return toG(fin[size_t(q) * V + lin(x, y, z, nx, ny)], q); };
        const uint32_t seed = g_dither_seed + uint32_t(t % 32);
        auto           storeg = [&](int x, int y, int z, int q, float g) {
            const size_t i = lin(x, y, z, nx, ny);
            fout[size_t(q) * V + i] = fromG(g, q, i, seed);
        };
        auto     wall = [&](int cls, int q) -> double { return cls == movingWall ? g_wall[1][q] : g_wall[0][q]; };
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int z = 0; z < nz; z++) bgk_step_shifted<Q>(nx, ny, nz, flag, omega, loadg, storeg, wall, z, z + 1, &g_zh);
    }
}

}  // namespace

extern "C" {

int orc_version() { return 3; }

// Zou-He boundary values of the following runs: pressure nodes rho, velocity nodes (ux, uy, uz).
// F16SR: seed of the first step of the following runs (step t uses seed + t mod 32).
int orc_set_dither_seed(uint32_t seed)
{
    g_dither_seed = seed;
    return 0;
}

// IEEE binary16 stochastic-rounding store of n values (the random bits given).
void orc_f32_to_f16_sr(const float* in, const uint32_t* r, uint16_t* out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = f32_to_f16_sr(in[i], r[i]);
}
void orc_dither_bits(const uint64_t* cell, const int32_t* q, uint32_t seed, uint32_t* out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = dither_bits(cell[i], q[i], seed);
}

int orc_set_zouhe(double rho, double ux, double uy, double uz)
{
    g_zh.rho = rho;
    g_zh.u[0] = ux, g_zh.u[1] = uy, g_zh.u[2] = uz;
    return 0;
}

int orc_max_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Cavity populations (RunCavityTwoPop.cu:159-206) in the requested storage.
// f16off/bf16off hold g = f - w on fluid nodes and the unshifted wall term on
// wall nodes is NOT stored (wall terms come from the wall table instead): wall
// nodes hold g = 0 there.
int orc_cavity_init(int nx, int ny, int nz, int Q, int storage, double ulb, void* pop)
{
    const size_t V = size_t(nx) * ny * nz;
    if (storage == ST_F64) {
        cavity_init_populations<double>(nx, ny, nz, Q, ulb, static_cast<double*>(pop));
    } else if (storage == ST_F32) {
        cavity_init_populations<float>(nx, ny, nz, Q, ulb, static_cast<float*>(pop));
    } else {
        uint16_t* p = static_cast<uint16_t*>(pop);
        for (size_t i = 0; i < size_t(Q) * V; i++) p[i] = 0;  // g = 0 <=> f = w
    }
    return 0;
}

// Classification + wall mask, packed.
int orc_cavity_flags(int nx, int ny, int nz, int Q, uint32_t* packed)
{
    const size_t          V = size_t(nx) * ny * nz;
    std::vector<CellType> f(V);
    cavity_init_flags(nx, ny, nz, f.data());
    compute_wall_mask(nx, ny, nz, Q, f.data());
    for (size_t i = 0; i < V; i++) packed[i] = pack(f[i]);
    return 0;
}

// Recomputes the wall mask from the classifications in `packed` (in place).
int orc_wall_mask(int nx, int ny, int nz, int Q, uint32_t* packed)
{
    const size_t          V = size_t(nx) * ny * nz;
    std::vector<CellType> f(V);
    for (size_t i = 0; i < V; i++) f[i] = unpack(packed[i]);
    compute_wall_mask(nx, ny, nz, Q, f.data());
    for (size_t i = 0; i < V; i++) packed[i] = pack(f[i]);
    return 0;
}

// wall: 4 x 27 doubles, wall term by classification of the wall node and population.
// mode CM_REFERENCE: the reference's unrolled D3Q19 arithmetic (storage f64/f32 only,
// compute type = storage type). CM_GENERIC: the per-direction BGK in the compute type
// (0 = double, 1 = float), any storage. Runs `steps` steps ping-ponging a <-> b;
// after an odd number of steps the result is in b.
int orc_lbm_run(int nx, int ny, int nz, int Q, int storage, int mode, int compute_float, double omega,
                const double* wall, const uint32_t* packed, void* a, void* b, int steps, int threads)
{
    const size_t V = size_t(nx) * ny * nz;
    if (threads <= 0) threads = orc_max_threads();
    std::vector<CellType> flag(V);
    for (size_t i = 0; i < V; i++) flag[i] = unpack(packed[i]);
    for (int c = 0; c < 4; c++)
        for (int q = 0; q < 27; q++) g_wall[c][q] = wall ? wall[c * 27 + q] : 0.0;

    if (mode == CM_REFERENCE) {
        if (Q != 19) return -1;
        for (int t = 0; t < steps; t++) {
            if (storage == ST_F64) {
                const double* fin = static_cast<const double*>(t % 2 == 0 ? a : b);
                double*       fout = static_cast<double*>(t % 2 == 0 ? b : a);
#pragma omp parallel for schedule(static) num_threads(threads)
                for (int z = 0; z < nz; z++)
                    d3q19_step<double, double>(nx, ny, nz, fin, fout, flag.data(), omega, z, z + 1, &g_zh, g_wall);
            } else if (storage == ST_F32) {
                const float* fin = static_cast<const float*>(t % 2 == 0 ? a : b);
                float*       fout = static_cast<float*>(t % 2 == 0 ? b : a);
                const float  om = float(omega);
#pragma omp parallel for schedule(static) num_threads(threads)
                for (int z = 0; z < nz; z++)
                    d3q19_step<float, float>(nx, ny, nz, fin, fout, flag.data(), om, z, z + 1, &g_zh, g_wall);
            } else {
                return -2;
            }
        }
        return 0;
    }

    if (mode == CM_SHIFTED) {
        const float om = float(omega);
        auto        go = [&](auto qTag) {
            constexpr int QQ = decltype(qTag)::value;
            if (storage == ST_F32) {
                shifted_run<QQ>(nx, ny, nz, flag.data(), om, static_cast<float*>(a), static_cast<float*>(b), steps,
                                [](float v, int q) { return v - float(weight(QQ, q)); },
                                [](float g, int q, size_t, uint32_t) { return float(weight(QQ, q)) + g; }, threads);
            } else if (storage == ST_F16OFF) {
                shifted_run<QQ>(nx, ny, nz, flag.data(), om, static_cast<uint16_t*>(a), static_cast<uint16_t*>(b), steps,
                                [](uint16_t v, int) { return f16_to_f32(v) * kF16Down; },
                                [](float g, int, size_t, uint32_t) { return f32_to_f16(g * kF16Up); },
                                threads);
            } else if (storage == ST_F16SR) {
                shifted_run<QQ>(nx, ny, nz, flag.data(), om, static_cast<uint16_t*>(a), static_cast<uint16_t*>(b), steps,
                                [](uint16_t v, int) { return f16_to_f32(v) * kF16Down; },
                                [](float g, int q, size_t i, uint32_t seed) { return f32_to_f16_sr(g * kF16Up, dither_bits(i, q, seed)); },
                                threads);
            } else if (storage == ST_BF16OFF) {
                shifted_run<QQ>(nx, ny, nz, flag.data(), om, static_cast<uint16_t*>(a), static_cast<uint16_t*>(b), steps,
                                [](uint16_t v, int) { return bf16_to_f32(v); },
                                [](float g, int, size_t, uint32_t) { return f32_to_bf16(g); }, threads);
            }
        };
        if (storage == ST_F64) return -2;
        if (Q == 19)
            go(std::integral_constant<int, 19>{});
        else
            go(std::integral_constant<int, 27>{});
        return 0;
    }

    auto run = [&](auto cTag) {
        using C = decltype(cTag);
        auto go = [&](auto qTag) {
            constexpr int QQ = decltype(qTag)::value;
            if (storage == ST_F64) {
                generic_run<C, QQ>(nx, ny, nz, flag.data(), omega, static_cast<double*>(a), static_cast<double*>(b), steps,
                                   [](double v, int) { return C(v); }, [](C v, int) { return double(v); }, threads);
            } else if (storage == ST_F32) {
                generic_run<C, QQ>(nx, ny, nz, flag.data(), omega, static_cast<float*>(a), static_cast<float*>(b), steps,
                                   [](float v, int) { return C(v); }, [](C v, int) { return float(v); }, threads);
            } else if (storage == ST_F16OFF) {
                generic_run<C, QQ>(nx, ny, nz, flag.data(), omega, static_cast<uint16_t*>(a), static_cast<uint16_t*>(b), steps,
                                   [](uint16_t v, int q) { return C(f16_to_f32(v) * kF16Down) + C(float(weight(QQ, q))); },
                                   [](C v, int q) { return f32_to_f16(float(v - C(float(weight(QQ, q)))) * kF16Up); }, threads);
            } else {
                generic_run<C, QQ>(nx, ny, nz, flag.data(), omega, static_cast<uint16_t*>(a), static_cast<uint16_t*>(b), steps,
                                   [](uint16_t v, int q) { return C(bf16_to_f32(v)) + C(float(weight(QQ, q))); },
                                   [](C v, int q) { return f32_to_bf16(float(v - C(float(weight(QQ, q))))); }, threads);
            }
        };
        if (Q == 19)
            go(std::integral_constant<int, 19>{});
        else
            go(std::integral_constant<int, 27>{});
    };
    if (Q != 19 && Q != 27) return -1;
    if (compute_float)
        run(float{});
    else
        run(double{});
    return 0;
}

// Density (V, may be NULL) and velocity (3 x V, SoA) as computeRhoAndU
// (LbmTools.h:383-437); wall = 4 x 27 wall terms by classification.
int orc_velocity(int nx, int ny, int nz, int Q, int storage, const double* wall, const uint32_t* packed, const void* pop,
                 double* rho, double* u)
{
    const size_t          V = size_t(nx) * ny * nz;
    std::vector<CellType> flag(V);
    for (size_t i = 0; i < V; i++) flag[i] = unpack(packed[i]);
    auto wt = [&](int cls, int q) -> double { return wall ? wall[(cls == movingWall ? 1 : 0) * 27 + q] : 0.0; };
    auto load = [&](int x, int y, int z, int q) -> double {
        const size_t i = size_t(q) * V + lin(x, y, z, nx, ny);
        switch (storage) {
            case ST_F64: return static_cast<const double*>(pop)[i];
            case ST_F32: return static_cast<const float*>(pop)[i];
            case ST_F16OFF:
            case ST_F16SR:
                return double(f16_to_f32(static_cast<const uint16_t*>(pop)[i]) * kF16Down) + double(float(weight(Q, q)));
            default: return double(bf16_to_f32(static_cast<const uint16_t*>(pop)[i])) + double(float(weight(Q, q)));
        }
    };
    rho_u_field(nx, ny, nz, Q, flag.data(), load, wt, rho, u);
    return 0;
}

// Time one reference-arithmetic D3Q19 FP32 step sample: returns microseconds.
double orc_time_d3q19_f32(int nx, int ny, int nz, int steps, int threads, double omega, const uint32_t* packed, float* a, float* b)
{
    auto t0 = std::chrono::steady_clock::now();
    orc_lbm_run(nx, ny, nz, 19, ST_F32, CM_REFERENCE, 1, omega, nullptr, packed, a, b, steps, threads);
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double, std::micro>(t1 - t0).count();
}

// ------------------------------------------------------------------ f16 / bf16 helpers
void orc_f32_to_f16(const float* in, uint16_t* out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = f32_to_f16(in[i]);
}
void orc_f16_to_f32(const uint16_t* in, float* out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = f16_to_f32(in[i]);
}
void orc_f32_to_bf16(const float* in, uint16_t* out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = f32_to_bf16(in[i]);
}
void orc_bf16_to_f32(const uint16_t* in, float* out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = bf16_to_f32(in[i]);
}

// ------------------------------------------------------------------ bGrid
// Two calls: with capacity 0 returns the block count; then fills the arrays.
int64_t orc_bgrid_build(int nx, int ny, int nz, const uint8_t* active, int32_t* origin, uint32_t* mask, uint32_t* conn,
                        int64_t capacity, uint64_t* n_active_voxels)
{
    BGrid g = bgrid_build(nx, ny, nz, active);
    if (n_active_voxels) *n_active_voxels = g.nActiveVoxels;
    if (capacity <= 0) return g.nBlocks;
    if (capacity < int64_t(g.nBlocks)) return -1;
    std::memcpy(origin, g.origin.data(), g.origin.size() * 4);
    std::memcpy(mask, g.mask.data(), g.mask.size() * 4);
    std::memcpy(conn, g.conn.data(), g.conn.size() * 4);
    return g.nBlocks;
}

// TestData::laplace on a dense int64 array; valid = inside the box and active[] != 0
// (active may be null: the full box).
int orc_laplace_i64(int nx, int ny, int nz, const uint8_t* active, const int64_t* a, int64_t* b)
{
    auto valid = [&](int x, int y, int z) {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return false;
        return active ? active[plin(x, y, z, nx, ny)] != 0 : true;
    };
    testdata_laplace<int64_t>(nx, ny, nz, a, b, valid);
    return 0;
}

void orc_masked_values_i64(int nx, int ny, int nz, int64_t offset, int digit, int64_t* out)
{
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) out[plin(x, y, z, nx, ny)] = masked_value<int64_t>(x, y, z, 0, offset, digit);
}

// ------------------------------------------------------------------ flow-over-sphere geometry
// Restatement of the geometry of ngb_geometry_sphere_tube (a project case,
// no reference counterpart): same double-precision expressions, same
// std::mt19937_64 stream and 53-bit uniforms.
int orc_sphere_tube(int nx, int ny, int nz, int ctrl_dx, const double* sc, double r, double band, const double* tc, double tr,
                    double tband, double amplitude, uint64_t seed, uint8_t* active, uint8_t* cls)
{
    const int           n_ctrl = nx / ctrl_dx + 2;
    std::vector<double> cy(n_ctrl), cz(n_ctrl);
    std::mt19937_64     rng(seed);
    for (int c = 0; c < n_ctrl; c++) {
        cy[c] = tc[0] + amplitude * (2.0 * u01(rng) - 1.0);
        cz[c] = tc[1] + amplitude * (2.0 * u01(rng) - 1.0);
    }
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const double dx = double(x) - sc[0], dy = double(y) - sc[1], dz = double(z) - sc[2];
                const double d2 = dx * dx + dy * dy + dz * dz;
                const double rs = r + band;
                bool         act = d2 <= rs * rs;
                const int    seg = x / ctrl_dx;
                const double t = double(x - seg * ctrl_dx) / double(ctrl_dx);
                const double ay = cy[seg] + t * (cy[seg + 1] - cy[seg]);
                const double az = cz[seg] + t * (cz[seg + 1] - cz[seg]);
                const double ty = double(y) - ay, tz = double(z) - az;
                const double rt = tr + tband;
                act = act || (ty * ty + tz * tz <= rt * rt);
                int c = undefined;
                if (act) c = d2 <= r * r ? bounceBack : (x == 0 ? movingWall : (x == nx - 1 ? outlet : bulk));
                const size_t i = lin(x, y, z, nx, ny);
                active[i] = act ? 1 : 0;
                cls[i] = uint8_t(c);
            }
    return 0;
}

// Packed flags (mask computed) from a dense uint8 class map.
int orc_flags_from_classes(int nx, int ny, int nz, int Q, const uint8_t* cls, uint32_t* packed)
{
    const size_t          V = size_t(nx) * ny * nz;
    std::vector<CellType> f(V);
    for (size_t i = 0; i < V; i++) f[i].classification = cls[i], f[i].wallNghBitflag = 0;
    compute_wall_mask(nx, ny, nz, Q, f.data());
    for (size_t i = 0; i < V; i++) packed[i] = pack(f[i]);
    return 0;
}

// ------------------------------------------------------------------ eGrid
// eGrid of one partition (eGrid_imp.h:8-129 -> Partitioner1D at block size 1):
// elements are the active cells in z, y, x order (SpanClassifier.h:228-237);
// origin = the cell (Partitioner1D.h:212-255); conn[s * count + e] = element at
// origin + points[s] or -1 (Partitioner1D.h:338-380, ePartition_imp.h isValidNgh).
// Returns the element count; origin / conn are written when non-null.
int64_t orc_egrid_build(int nx, int ny, int nz, const uint8_t* active, const int8_t* points, int npts, int32_t* origin, int32_t* conn)
{
    const size_t         V = size_t(nx) * ny * nz;
    std::vector<int32_t> elem(V, -1);
    int64_t              count = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const size_t i = lin(x, y, z, nx, ny);
                if (!active[i]) continue;
                elem[i] = int32_t(count);
                if (origin) {
                    origin[3 * count] = x;
                    origin[3 * count + 1] = y;
                    origin[3 * count + 2] = z;
                }
                count++;
            }
    if (conn) {
        int64_t e = 0;
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    if (!active[lin(x, y, z, nx, ny)]) continue;
                    for (int s = 0; s < npts; s++) {
                        const int xx = x + points[3 * s], yy = y + points[3 * s + 1], zz = z + points[3 * s + 2];
                        int32_t   v = -1;
                        if (xx >= 0 && yy >= 0 && zz >= 0 && xx < nx && yy < ny && zz < nz) v = elem[lin(xx, yy, zz, nx, ny)];
                        conn[int64_t(s) * count + e] = v;
                    }
                    e++;
                }
    }
    return count;
}

// ------------------------------------------------------------------ Poisson
void orc_box_boundary(int nx, int ny, int nz, int8_t* bd) { box_boundary(nx, ny, nz, bd); }

void orc_gaussian_sources(int nx, int ny, int nz, uint64_t seed, double* centres, double* amps)
{
    gaussian_sources(nx, ny, nz, seed, centres, amps);
}

int orc_laplacian_f64(int nx, int ny, int nz, double h, const double* u, const int8_t* bd, double* out)
{
    laplacian_apply<double, double>(nx, ny, nz, h, u, bd, out);
    return 0;
}
int orc_laplacian_f32(int nx, int ny, int nz, double h, const float* u, const int8_t* bd, float* out)
{
    laplacian_apply<float, float>(nx, ny, nz, h, u, bd, out);
    return 0;
}

// Mixed-precision Jacobi-PCG (the GPU algorithm). result[0] = iterations,
// result[1] = converged, result[2] = relative true residual, result[3] = refreshes.
int orc_pcg_f32(int nx, int ny, int nz, double h, const int8_t* bd, const float* b, double* x, double tol, int max_iter,
                int refresh_every, double* result, int jacobi)
{
    PcgOracle<float> s(nx, ny, nz, h, bd, jacobi != 0);
    PcgResult        r = s.solve(b, x, tol, max_iter, refresh_every);
    result[0] = r.iterations;
    result[1] = r.converged;
    result[2] = r.rel_residual;
    result[3] = r.refreshes;
    return 0;
}
int orc_pcg_f64(int nx, int ny, int nz, double h, const int8_t* bd, const double* b, double* x, double tol, int max_iter,
                int refresh_every, double* result, int jacobi)
{
    PcgOracle<double> s(nx, ny, nz, h, bd, jacobi != 0);
    PcgResult         r = s.solve(b, x, tol, max_iter, refresh_every);
    result[0] = r.iterations;
    result[1] = r.converged;
    result[2] = r.rel_residual;
    result[3] = r.refreshes;
    return 0;
}

double orc_reference_cg_f64(int nx, int ny, int nz, double h, const int8_t* bd, const double* b, double* x, int iters)
{
    return reference_cg<double>(nx, ny, nz, h, bd, b, x, iters);
}
double orc_reference_cg_f32(int nx, int ny, int nz, double h, const int8_t* bd, const float* b, float* x, int iters)
{
    return reference_cg<float>(nx, ny, nz, h, bd, b, x, iters);
}

}  // extern "C"
