// ORACLE — test infrastructure only.
//
// CPU restatement of Neon's 7-point Laplacian matvec and of the libNeonSolver
// conjugate-gradient iteration, plus the mixed-precision Jacobi-PCG that the
// GPU solver implements (FP32 fields, FP64 reductions, FP64 solution with a
// periodic true-residual refresh). Used by tests as the checker.
//
// Follows (paths relative to the Neon repository):
//   libNeonSolver/src/linear/matvecs/LaplacianMatVec.cu:23-95
//       Fixed rows are the identity; Free rows (n_valid u - sum of valid neighbours) / h^2
//   libNeonSolver/src/linear/krylov/CGContainers.cu:44-149
//       initR, AXPY, updateXandR (alpha = delta_new / pAp), updateP (beta = 0 on the first pass)
//   libNeonSolver/src/linear/krylov/CG.cpp:26-145   the iteration order
//   libNeonSolver/include/Neon/solver/linear/IterativeLinearSolver.h:17-21
//       BoundaryCondition { Fixed = 0, Free = 1 }
//   libNeonDomain/include/Neon/domain/tools/TestData.h:412-443
//       the integer "laplace" known-answer operator b = a - count * sum(valid neighbours)
//   libNeonDomain/include/Neon/domain/tools/IODomain.h:236-250
//       the "masked" initial values z + y 10^d + x 10^2d + c 10^3d + offset 10^(3d+1)
#pragma once
#include <cstdint>
#include <cmath>
#include <vector>
#include <random>
#include <limits>
#include <type_traits>

namespace oracle {

enum BoundaryCondition : int8_t { Fixed = 0, Free = 1 };

inline size_t plin(int x, int y, int z, int nx, int ny) { return size_t(x) + size_t(nx) * (size_t(y) + size_t(ny) * size_t(z)); }

// Neighbour validity of a single-partition dGrid (dPartition.h:228-263): inside [0, dim).
template <typename T, typename Acc = T>
void laplacian_apply(int nx, int ny, int nz, double h, const T* u, const int8_t* bd, T* out)
{
    const Acc invh2 = Acc(1.0) / (Acc(h) * Acc(h));
    static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const size_t i = plin(x, y, z, nx, ny);
                const Acc    c = Acc(u[i]);
                if (bd[i] == Fixed) {
                    out[i] = T(c);
                    continue;
                }
                Acc sum = 0;
                int n = 0;
                for (auto& o : off) {
                    const int X = x + o[0], Y = y + o[1], Z = z + o[2];
                    if (X < 0 || Y < 0 || Z < 0 || X >= nx || Y >= ny || Z >= nz) continue;
                    sum += Acc(u[plin(X, Y, Z, nx, ny)]);
                    n++;
                }
                out[i] = T((-sum + Acc(n) * c) * invh2);
            }
}

// TestData::laplace: b = a - count * sum over valid 6-neighbours (integer exact).
// valid(x,y,z) says whether a voxel exists (dGrid: inside the box; bGrid: active).
template <typename T, typename Valid>
void testdata_laplace(int nx, int ny, int nz, const T* a, T* b, Valid valid)
{
    static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                if (!valid(x, y, z)) continue;
                T   res = 0;
                int count = 0;
                for (auto& o : off) {
                    const int X = x + o[0], Y = y + o[1], Z = z + o[2];
                    if (!valid(X, Y, Z)) continue;
                    res += a[plin(X, Y, Z, nx, ny)];
                    count++;
                }
                b[plin(x, y, z, nx, ny)] = a[plin(x, y, z, nx, ny)] - T(count) * res;
            }
}

template <typename T>
T masked_value(int x, int y, int z, int c, T offset, int digit)
{
    T m = 1;
    for (int i = 0; i < digit; i++) m *= 10;
    return T(z) + T(y) * m + T(x) * m * m + T(c) * m * m * m + offset * m * m * m * 10;
}

// ------------------------------------------------------------------ problem set-up
// Zero Dirichlet box: every face cell is Fixed (u = 0), the rest Free.
inline void box_boundary(int nx, int ny, int nz, int8_t* bd)
{
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const bool face = x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1;
                bd[plin(x, y, z, nx, ny)] = face ? Fixed : Free;
            }
}

// Deterministic uniform in [0,1) from a 64-bit Mersenne Twister draw (53 bits).
inline double u01(std::mt19937_64& g) { return double(g() >> 11) * (1.0 / 9007199254740992.0); }

// Eight Gaussians: centres uniform in [N/8, 7N/8) per axis, amplitudes uniform in [-1, 1).
inline void gaussian_sources(int nx, int ny, int nz, uint64_t seed, double* centres /*8x3*/, double* amps /*8*/)
{
    std::mt19937_64 g(seed);
    for (int k = 0; k < 8; k++) {
        centres[3 * k + 0] = nx / 8.0 + u01(g) * (0.75 * nx);
        centres[3 * k + 1] = ny / 8.0 + u01(g) * (0.75 * ny);
        centres[3 * k + 2] = nz / 8.0 + u01(g) * (0.75 * nz);
        amps[k] = 2.0 * u01(g) - 1.0;
    }
}

// ------------------------------------------------------------------ mixed-precision Jacobi-PCG
// The algorithm of the GPU solver, step for step:
//   fields r, p, s, x_lo in T; x_hi and every reduction in double;
//   z = invdiag * r with invdiag = h^2 / n_valid on Free rows and 1 on Fixed rows;
//   pass A: beta = (rz_prev == 0 ? 0 : rz / rz_prev); p = z + beta p; s = A p; alpha = rz / <p,s>
//   pass B: x_lo += alpha p; r -= alpha s; rz_prev = rz; rz = <r,z>; rr = <r,r>
//   refresh when (it+1) % refresh_every == 0 or sqrt(rr)/|b| <= tol:
//           x_hi += x_lo; x_lo = 0; r = T(b - A x_hi) (double); rz = <r,z>;
//           converged iff |b - A x_hi| / |b| <= tol.
//   T = float (the GPU's cg_refresh_ff_kernel): the true residual b - A x_hi
//   is kept as a float pair (hi, lo) from the start, and a refresh subtracts
//   A x_lo from it in float-pair arithmetic (TwoSum, TwoProduct by fma, the
//   neighbours in the order +x, -x, +y, -y, +z, -z, 1/h^2 as a float pair)
//   before x_lo is folded into x_hi; r = hi, |b - A x_hi| from hi.
struct PcgResult {
    int    iterations = 0;
    bool   converged = false;
    double rel_residual = 0;
    int    refreshes = 0;
};

template <typename T>
struct PcgOracle {
    int                 nx, ny, nz;
    double              h;
    std::vector<int8_t> bd;
    std::vector<T>      invdiag;

    PcgOracle(int nx_, int ny_, int nz_, double h_, const int8_t* bd_, bool jacobi = true) : nx(nx_), ny(ny_), nz(nz_), h(h_), bd(bd_, bd_ + size_t(nx_) * ny_ * nz_)
    {
        invdiag.resize(bd.size());
        static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    const size_t i = plin(x, y, z, nx, ny);
                    if (bd[i] == Fixed || !jacobi) {
                        invdiag[i] = T(1);
                        continue;
                    }
                    int n = 0;
                    for (auto& o : off) {
                        const int X = x + o[0], Y = y + o[1], Z = z + o[2];
                        if (X >= 0 && Y >= 0 && Z >= 0 && X < nx && Y < ny && Z < nz) n++;
                    }
                    invdiag[i] = T(h * h / double(n));
                }
    }

    // b - A x in double for every cell (0 on Fixed rows).
    void true_residual(const T* b, const double* x, double* res) const
    {
        const size_t        V = bd.size();
        std::vector<double> ax(V);
        laplacian_apply<double, double>(nx, ny, nz, h, x, bd.data(), ax.data());
        for (size_t i = 0; i < V; i++) res[i] = bd[i] == Fixed ? 0.0 : double(b[i]) - ax[i];
    }

    // Float-pair helpers (the GPU's FF arithmetic, IEEE single, no contraction).
    struct FF {
        float hi, lo;
    };
    static FF two_sum(float a, float b)
    {
        const float s = a + b, bb = s - a;
        return FF{s, (a - (s - bb)) + (b - bb)};
    }
    static FF ff_norm(float hi, float lo)
    {
        const float s = hi + lo;
        return FF{s, lo - (s - hi)};
    }
    static FF ff_add(FF a, float b)
    {
        const FF t = two_sum(a.hi, b);
        return ff_norm(t.hi, t.lo + a.lo);
    }

    // rt -= A x_lo on Free cells (float pair); returns the new high part (0 on Fixed cells).
    float ff_refresh_cell(int x, int y, int z, const std::vector<float>& xlo, float& rt_hi, float& rt_lo, float ih_hi,
                          float ih_lo) const
    {
        const size_t i = plin(x, y, z, nx, ny);
        if (bd[i] == Fixed) return 0.f;
        static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        int              n = 0;
        for (auto& o : off) {
            const int X = x + o[0], Y = y + o[1], Z = z + o[2];
            if (X >= 0 && Y >= 0 && Z >= 0 && X < nx && Y < ny && Z < nz) n++;
        }
        const float xc = xlo[i];
        const float pp = float(n) * xc;
        FF          a{pp, std::fma(float(n), xc, -pp)};
        for (auto& o : off) {
            const int X = x + o[0], Y = y + o[1], Z = z + o[2];
            if (X >= 0 && Y >= 0 && Z >= 0 && X < nx && Y < ny && Z < nz) a = ff_add(a, -xlo[plin(X, Y, Z, nx, ny)]);
        }
        const float ph = a.hi * ih_hi;
        const float pl = std::fma(a.hi, ih_hi, -ph) + (a.hi * ih_lo + a.lo * ih_hi);
        const FF    t = two_sum(rt_hi, -ph);
        const FF    rt = ff_norm(t.hi, t.lo + (rt_lo - pl));
        rt_hi = rt.hi;
        rt_lo = rt.lo;
        return rt.hi;
    }

    PcgResult solve(const T* b, double* x_hi, double tol, int max_iter, int refresh_every) const
    {
        constexpr bool      kFF = std::is_same<T, float>::value;
        const size_t        V = bd.size();
        std::vector<T>      r(V), p(V, T(0)), s(V), xlo(V, T(0));
        std::vector<double> tr(V);
        std::vector<float>  rt_hi(kFF ? V : 0), rt_lo(kFF ? V : 0);
        const double        ih2 = 1.0 / (h * h);
        const float         ih_hi = float(ih2), ih_lo = float(ih2 - double(ih_hi));
        double              bnorm2 = 0;
        for (size_t i = 0; i < V; i++)
            if (bd[i] == Free) bnorm2 += double(b[i]) * double(b[i]);
        const double bnorm = std::sqrt(bnorm2);
        PcgResult    res;
        true_residual(b, x_hi, tr.data());
        double rz = 0, rr = 0;
        for (size_t i = 0; i < V; i++) {
            r[i] = T(tr[i]);
            rz += double(r[i]) * double(T(invdiag[i] * r[i]));
            rr += tr[i] * tr[i];
            if constexpr (kFF) {
                rt_hi[i] = float(tr[i]);
                rt_lo[i] = float(tr[i] - double(rt_hi[i]));
            }
        }
        res.rel_residual = bnorm > 0 ? std::sqrt(rr) / bnorm : 0.0;
        if (bnorm == 0 || res.rel_residual <= tol) {
            res.converged = true;
            return res;
        }
        double rz_prev = 0;
        for (int it = 0; it < max_iter; it++) {
            // pass A
            const double beta = rz_prev == 0 ? 0.0 : rz / rz_prev;
            for (size_t i = 0; i < V; i++) p[i] = T(invdiag[i] * r[i]) + T(beta) * p[i];
            laplacian_apply<T, T>(nx, ny, nz, h, p.data(), bd.data(), s.data());
            double pAp = 0;
            for (size_t i = 0; i < V; i++) pAp += double(p[i]) * double(s[i]);
            const double alpha = rz / pAp;
            // pass B
            double rz_new = 0;
            rr = 0;
            for (size_t i = 0; i < V; i++) {
                xlo[i] = xlo[i] + T(alpha) * p[i];
                r[i] = r[i] - T(alpha) * s[i];
                const T zi = T(invdiag[i] * r[i]);
                rz_new += double(r[i]) * double(zi);
                rr += double(r[i]) * double(r[i]);
            }
            rz_prev = rz;
            rz = rz_new;
            res.iterations = it + 1;
            const bool last = (it + 1) >= max_iter;
            const bool want = ((it + 1) % refresh_every == 0) || (std::sqrt(rr) / bnorm <= tol) || last;
            if (want) {
                res.refreshes++;
                rz = 0;
                double trr = 0;
                if constexpr (kFF) {
                    for (int z = 0; z < nz; z++)
                        for (int y = 0; y < ny; y++)
                            for (int x = 0; x < nx; x++) {
                                const size_t i = plin(x, y, z, nx, ny);
                                const float  rh = ff_refresh_cell(x, y, z, xlo, rt_hi[i], rt_lo[i], ih_hi, ih_lo);
                                r[i] = rh;
                                rz += double(rh) * double(float(invdiag[i] * rh));
                                trr += double(rh) * double(rh);
                            }
                    for (size_t i = 0; i < V; i++) {
                        x_hi[i] += double(xlo[i]);
                        xlo[i] = T(0);
                    }
                } else {
                    for (size_t i = 0; i < V; i++) {
                        x_hi[i] += double(xlo[i]);
                        xlo[i] = T(0);
                    }
                    true_residual(b, x_hi, tr.data());
                    for (size_t i = 0; i < V; i++) {
                        r[i] = T(tr[i]);
                        rz += double(r[i]) * double(T(invdiag[i] * r[i]));
                        trr += tr[i] * tr[i];
                    }
                }
                res.rel_residual = std::sqrt(trr) / bnorm;
                if (res.rel_residual <= tol) {
                    res.converged = true;
                    break;
                }
            }
        }
        return res;
    }
};

// ------------------------------------------------------------------ plain reference CG (CG.cpp:55-145)
// Fixed number of iterations of the libNeonSolver sequence in type T:
//   initR; s = A x; r -= s; delta = <r,r>; p = r;
//   loop: updateP (beta = 0 on the first pass, else delta_new / delta_old); s = A p; pAp = <p,s>;
//         alpha = delta_new / pAp; delta_old = delta_new; x += alpha p; r -= alpha s; delta_new = <r,r>
// Reductions run in double. Returns sqrt(delta_new) after the last iteration.
template <typename T>
double reference_cg(int nx, int ny, int nz, double h, const int8_t* bd, const T* b, T* x, int iters)
{
    const size_t   V = size_t(nx) * ny * nz;
    std::vector<T> r(V), s(V), p(V);
    for (size_t i = 0; i < V; i++) r[i] = bd[i] == Free ? b[i] : x[i];
    laplacian_apply<T, T>(nx, ny, nz, h, x, bd, s.data());
    double delta_new = 0;
    for (size_t i = 0; i < V; i++) {
        r[i] -= s[i];
        delta_new += double(r[i]) * double(r[i]);
    }
    for (size_t i = 0; i < V; i++) p[i] = r[i];
    double delta_old = 0;
    for (int it = 0; it < iters; it++) {
        const double beta = std::abs(delta_old) > double(std::numeric_limits<T>::epsilon()) ? delta_new / delta_old : 0.0;
        for (size_t i = 0; i < V; i++) p[i] = r[i] + T(beta) * p[i];
        laplacian_apply<T, T>(nx, ny, nz, h, p.data(), bd, s.data());
        double pAp = 0;
        for (size_t i = 0; i < V; i++) pAp += double(p[i]) * double(s[i]);
        const double alpha = delta_new / pAp;
        delta_old = delta_new;
        delta_new = 0;
        for (size_t i = 0; i < V; i++) {
            x[i] += T(alpha) * p[i];
            r[i] -= T(alpha) * s[i];
            delta_new += double(r[i]) * double(r[i]);
        }
    }
    return std::sqrt(delta_new);
}

}  // namespace oracle
