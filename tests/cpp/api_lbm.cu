// The lid-driven cavity of benchmarks/lbm-lid-driven-cavity-flow written
// against the GB300 Neon API, two ways:
//  (a) "user" — the application's own per-cell D3Q19 BGK lambda (pull with
//      half-way bounce-back, the reference's FP64 expression shapes) through
//      dGrid::newContainer + Loader::load(STENCIL) and two Skeletons that
//      alternate the population fields (LbmIteration.h:27-96);
//  (b) "gb300" — the same iteration through Neon::gb300::iteration (the
//      sm_103a kernel of the C ABI), on dGrid and on an all-active bGrid.
// FP64, N^3, `steps` steps; writes the newest populations (dense SoA, q
// slowest) to <outdir>/cavity_{user,gb300,bgrid}.bin.
#include <cstdio>
#include <fstream>

#include "Neon/Neon.h"
#include "Neon/domain/Grids.h"
#include "Neon/gb300/lbm.h"
#include "Neon/skeleton/Skeleton.h"

namespace {

constexpr int kC[19][3] = {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {-1, 0, 1},
                           {0, -1, -1}, {0, -1, 1}, {0, 0, 0},  {1, 0, 0},   {0, 1, 0},  {0, 0, 1},   {1, 1, 0},
                           {1, -1, 0},  {1, 0, 1},  {1, 0, -1}, {0, 1, 1},   {0, 1, -1}};
double w_of(int q) { return q == 9 ? 1. / 3. : ((q % 10) < 3 ? 1. / 18. : 1. / 36.); }

// (a): the application's container, written by the user in Neon's style.
template <typename PopField, typename FlagField>
Neon::set::Container userIteration(const PopField& fInField, const FlagField& flagField, double omega, PopField& fOutField)
{
    return fInField.getGrid().newContainer("LBM_iteration", [&, omega](Neon::set::Loader& L) {
        const auto& fIn = L.load(fInField, Neon::Pattern::STENCIL);
        auto&       fOut = L.load(fOutField);
        const auto& flag = L.load(flagField);
        return [=] NEON_CUDA_HOST_DEVICE(const typename PopField::Idx& i) mutable {
            const uint32_t f = flag(i, 0);
            if (NGB_FLAG_CLASS(f) != NGB_CELL_BULK) return;
            const uint32_t m = NGB_FLAG_MASK(f);
            double         p[19];
            // pull: population q comes from x - c_q; across a wall, the opposite
            // population of this cell plus the wall node's stored value
#define PULL(Q, GX, GY, GZ, O)                                                                                  \
    p[Q] = (m & (1u << Q)) ? fIn(i, O) + fIn.template getNghData<GX, GY, GZ>(i, O)() : fIn.template getNghData<GX, GY, GZ>(i, Q)();
            PULL(0, 1, 0, 0, 10) PULL(1, 0, 1, 0, 11) PULL(2, 0, 0, 1, 12) PULL(3, 1, 1, 0, 13) PULL(4, 1, -1, 0, 14)
            PULL(5, 1, 0, 1, 15) PULL(6, 1, 0, -1, 16) PULL(7, 0, 1, 1, 17) PULL(8, 0, 1, -1, 18)
            PULL(10, -1, 0, 0, 0) PULL(11, 0, -1, 0, 1) PULL(12, 0, 0, -1, 2) PULL(13, -1, -1, 0, 3) PULL(14, -1, 1, 0, 4)
            PULL(15, -1, 0, -1, 5) PULL(16, -1, 0, 1, 6) PULL(17, 0, -1, -1, 7) PULL(18, 0, -1, 1, 8)
#undef PULL
            p[9] = fIn(i, 9);
            const double xm = p[0] + p[3] + p[4] + p[5] + p[6];
            const double xp = p[10] + p[13] + p[14] + p[15] + p[16];
            const double x0 = p[9] + p[1] + p[2] + p[7] + p[8] + p[11] + p[12] + p[17] + p[18];
            const double ym = p[1] + p[3] + p[7] + p[8] + p[14];
            const double yp = p[4] + p[11] + p[13] + p[17] + p[18];
            const double zm = p[2] + p[5] + p[7] + p[16] + p[18];
            const double zp = p[6] + p[8] + p[12] + p[15] + p[17];
            const double rho = xm + xp + x0;
            const double u0 = (xp - xm) / rho, u1 = (yp - ym) / rho, u2 = (zp - zm) / rho;
            const double usqr = 1.5 * (u0 * u0 + u1 * u1 + u2 * u2);
            const double cu[9] = {u0, u1, u2, u0 + u1, u0 - u1, u0 + u2, u0 - u2, u1 + u2, u1 - u2};
            for (int k = 0; k < 9; k++) {
                const double wk = k < 3 ? (1. / 18.) : (1. / 36.);
                const double eq = rho * wk * (1. - 3. * cu[k] + 4.5 * cu[k] * cu[k] - usqr);
                const double eqo = eq + rho * wk * 6. * cu[k];
                fOut(i, k) = (1. - omega) * p[k] + omega * eq;
                fOut(i, k + 10) = (1. - omega) * p[k + 10] + omega * eqo;
            }
            fOut(i, 9) = (1. - omega) * p[9] + omega * (rho * (1. / 3.) * (1. - usqr));
        };
    });
}

template <typename Grid>
void initCavity(typename Grid::template Field<double, 19>& pop, typename Grid::template Field<uint32_t, 1>& flags, int N, double ulb)
{
    auto face = [N](const Neon::index_3d& p) { return p.x == 0 || p.x == N - 1 || p.y == 0 || p.y == N - 1 || p.z == 0 || p.z == N - 1; };
    pop.forEachActiveCell([&](const Neon::index_3d& p, int q, double& v) {
        v = w_of(q);
        if (face(p)) v = p.y == N - 1 ? -6. * w_of(q) * ulb * kC[q][0] : 0.0;  // RunCavityTwoPop.cu:168-186
    });
    flags.forEachActiveCell([&](const Neon::index_3d& p, int, uint32_t& f) {
        f = NGB_MAKE_FLAG(0, face(p) ? (p.y == N - 1 ? NGB_CELL_MOVINGWALL : NGB_CELL_BOUNCEBACK) : NGB_CELL_BULK);
    });
    pop.updateDeviceData(0);
    flags.updateDeviceData(0);
}

template <typename Grid>
void dump(const std::string& path, typename Grid::template Field<double, 19>& f, int N)
{
    const size_t        V = size_t(N) * N * N;
    std::vector<double> dense(19 * V, 0.0);
    f.forEachActiveCell([&](const Neon::index_3d& p, int q, double& v) { dense[q * V + p.x + size_t(N) * (p.y + size_t(N) * p.z)] = v; });
    std::ofstream o(path, std::ios::binary);
    o.write(reinterpret_cast<const char*>(dense.data()), dense.size() * sizeof(double));
}

template <typename Grid, bool User>
void cavity(const std::string& path, int N, int steps, double ulb, double Re)
{
    Neon::Backend bk(std::vector<int>{0}, Neon::Runtime::stream);
    std::vector<Neon::index_3d> stencil;
    for (auto& c : kC) stencil.push_back(Neon::index_3d(c[0], c[1], c[2]));
    Grid grid(bk, {N, N, N}, [](const Neon::index_3d&) { return true; }, stencil);
    auto pop0 = grid.template newField<double, 19>("Population", 19, 0.0);
    auto pop1 = grid.template newField<double, 19>("Population", 19, 0.0);
    auto flags = grid.template newField<uint32_t, 1>("Material", 1, 0u);
    initCavity<Grid>(pop0, flags, N, ulb);
    initCavity<Grid>(pop1, flags, N, ulb);
    Neon::gb300::computeWallNghMask<19>(flags).run(0);
    const double nu = ulb * double(N - 2) / Re;  // Config.cpp:105-111
    const double omega = 1. / (3. * nu + 0.5);
    Neon::gb300::WallTerms walls;
    for (int q = 0; q < 19; q++) walls.movingWall[q] = -6. * w_of(q) * ulb * kC[q][0];
    Neon::skeleton::Skeleton sk[2] = {Neon::skeleton::Skeleton(bk), Neon::skeleton::Skeleton(bk)};
    if constexpr (User) {
        sk[0].sequence(std::vector<Neon::set::Container>{userIteration(pop0, flags, omega, pop1)}, "LBM_iteration_0");
        sk[1].sequence(std::vector<Neon::set::Container>{userIteration(pop1, flags, omega, pop0)}, "LBM_iteration_1");
    } else {
        sk[0].sequence(std::vector<Neon::set::Container>{Neon::gb300::iteration<19>(pop0, flags, omega, walls, pop1)}, "LBM_iteration_0");
        sk[1].sequence(std::vector<Neon::set::Container>{Neon::gb300::iteration<19>(pop1, flags, omega, walls, pop0)}, "LBM_iteration_1");
    }
    for (int t = 0; t < steps; t++) sk[t % 2].run();
    auto& out = steps % 2 == 0 ? pop0 : pop1;
    out.updateHostData(0);
    bk.sync(0);
    dump<Grid>(path, out, N);
    std::printf("%s ok\n", path.c_str());
}

}  // namespace

int main(int argc, char** argv)
{
    const std::string outdir = argc > 1 ? argv[1] : ".";
    const int         N = 24, steps = 60;
    cavity<Neon::dGrid, true>(outdir + "/cavity_user.bin", N, steps, 0.1, 100.0);
    cavity<Neon::dGrid, false>(outdir + "/cavity_gb300.bin", N, steps, 0.1, 100.0);
    cavity<Neon::bGrid, false>(outdir + "/cavity_bgrid.bin", N, steps, 0.1, 100.0);
    cavity<Neon::bGrid, true>(outdir + "/cavity_bgrid_user.bin", N, steps, 0.1, 100.0);
    return 0;
}
