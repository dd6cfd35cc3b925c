// The Poisson app of Neon (apps/poisson/poisson.cu:8-167) solved with the
// learned-preconditioner sibling of CG_t, LearnedFCG_t, through the GB300
// Neon API: a dGrid, fields x, b and bd, LaplacianMatVec, solve(A, x, b, bd,
// params, result). Arguments: <outdir> <N> <weights file> <levels>. The
// right-hand side is read from <outdir>/poisson_b.bin (N^3 floats); the
// iteration count, residual and whether Jacobi-PCG took over are printed.
#include <cstdio>
#include <fstream>

#include "Neon/Neon.h"
#include "Neon/domain/dGrid.h"
#include "Neon/solver/linear/krylov/LearnedFCG.h"

int main(int argc, char** argv)
{
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s outdir N weights levels\n", argv[0]);
        return 2;
    }
    const std::string outdir = argv[1];
    const int         N = std::atoi(argv[2]);
    const std::string weights = argv[3];
    const int         levels = std::atoi(argv[4]);
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
    Neon::solver::LearnedFCG_t<Neon::dGrid, float> fcg(weights, levels);
    fcg.init(x);
    Neon::solver::SolverParams params;
    params.maxIterations = 2000;
    params.toleranceRel = 1e-8;
    Neon::solver::SolverResultInfo info;
    const auto status = fcg.solve(A, x, b, bd, params, info);
    std::printf("status=%d iterations=%zu residual=%.3e fallback=%d solve_ms=%.3f\n", int(status), info.numIterations,
                info.residualEnd, int(fcg.usedFallback()), info.solveTime);
    return status == Neon::solver::SolverStatus::Converged ? 0 : 1;
}
