// The Poisson app of Neon (apps/poisson/poisson.cu:8-167) written against the
// GB300 Neon API: a dGrid, fields x, b and the boundary field bd (faces Fixed,
// interior Free), LaplacianMatVec and CG_t::solve. The right-hand side is read
// from <outdir>/poisson_b.bin (N^3 floats); the solution is written to
// <outdir>/poisson_x.bin and the iteration count / residual printed.
#include <cstdio>
#include <fstream>

#include "Neon/Neon.h"
#include "Neon/domain/dGrid.h"
#include "Neon/solver/linear/krylov/CG.h"

int main(int argc, char** argv)
{
    const std::string outdir = argc > 1 ? argv[1] : ".";
    const int         N = argc > 2 ? std::atoi(argv[2]) : 40;
    const size_t      V = size_t(N) * N * N;
    std::vector<float> rhs(V);
    {
        std::ifstream in(outdir + "/poisson_b.bin", std::ios::binary);
        in.read(reinterpret_cast<char*>(rhs.data()), V * sizeof(float));
        if (!in) {
            std::fprintf(stderr, "cannot read poisson_b.bin\n");
            return 2;
        }
    }
    Neon::Backend bk(std::vector<int>{0}, Neon::Runtime::stream);
    Neon::dGrid   grid(bk, {N, N, N}, [](const Neon::index_3d&) { return true; }, Neon::domain::Stencil::s7_Laplace_t());
    auto          x = grid.newField<float, 0>("x", 1, 0.f);
    auto          b = grid.newField<float, 0>("b", 1, 0.f);
    auto          bd = grid.newField<int8_t, 0>("bd", 1, int8_t(0));
    b.forEachActiveCell([&](const Neon::index_3d& p, int, float& v) { v = rhs[p.x + size_t(N) * (p.y + size_t(N) * p.z)]; });
    bd.forEachActiveCell([&](const Neon::index_3d& p, int, int8_t& v) {
        const bool face = p.x == 0 || p.y == 0 || p.z == 0 || p.x == N - 1 || p.y == N - 1 || p.z == N - 1;
        v = face ? Neon::solver::Fixed : Neon::solver::Free;
    });
    b.updateDeviceData(0);
    bd.updateDeviceData(0);
    x.updateDeviceData(0);

    auto A = std::make_shared<Neon::solver::LaplacianMatVec<Neon::dGrid, float>>(1.0f);
    Neon::solver::CG_t<Neon::dGrid, float> cg;
    cg.init(x);
    Neon::solver::SolverParams params;
    params.maxIterations = 5000;
    params.toleranceRel = 1e-8;
    Neon::solver::SolverResultInfo info;
    const auto status = cg.solve(A, x, b, bd, params, info);

    // A x through the matVec container, to report |b - A x| / |b| in float
    auto Ax = grid.newField<float, 0>("Ax", 1, 0.f);
    A->matVec(x, bd, Ax).run(0);
    x.updateHostData(0);
    Ax.updateHostData(0);
    bk.sync(0);
    std::vector<float> xs(V);
    x.forEachActiveCell([&](const Neon::index_3d& p, int, float& v) { xs[p.x + size_t(N) * (p.y + size_t(N) * p.z)] = v; });
    std::ofstream o(outdir + "/poisson_x.bin", std::ios::binary);
    o.write(reinterpret_cast<const char*>(xs.data()), V * sizeof(float));
    std::printf("status=%d iterations=%zu residual=%.3e solve_ms=%.3f\n", int(status), info.numIterations, info.residualEnd,
                info.solveTime);
    return status == Neon::solver::SolverStatus::Converged ? 0 : 1;
}
