// The domain-stencil and skeleton-stencil tests of Neon
// (libNeonDomain/tests/domain-stencil/src/stencil.cu:11-205,
// libNeonSkeleton/tests/unit/skeleton-stencil/src/stencil.cu:18-127) written
// against the GB300 Neon API: integer 6-neighbour operator b = a - count *
// sum(valid neighbours) through grid.newContainer + Loader::load(STENCIL),
// once through Container::run and once through a Skeleton sequence.
// Writes dense int64 results to <outdir>/<grid>_<nx>x<ny>x<nz>_{run,skel}.bin.
#include <cstdio>
#include <fstream>

#include "Neon/Neon.h"
#include "Neon/domain/Grids.h"
#include "Neon/skeleton/Skeleton.h"

template <typename Field>
Neon::set::Container laplace(const Field& fieldA, Field& fieldB)
{
    const auto& grid = fieldA.getGrid();
    return grid.newContainer("stencilFun", [&](Neon::set::Loader& loader) {
        const auto a = loader.load(fieldA, Neon::Pattern::STENCIL);
        auto       b = loader.load(fieldB);
        return [=] NEON_CUDA_HOST_DEVICE(const typename Field::Idx& idx) mutable {
            using N = Neon::int8_3d;
            const N dirs[6] = {N(1, 0, 0), N(-1, 0, 0), N(0, 1, 0), N(0, -1, 0), N(0, 0, 1), N(0, 0, -1)};
            for (int c = 0; c < a.cardinality(); c++) {
                typename Field::Type partial = 0;
                int                  count = 0;
                for (const auto& d : dirs) {
                    auto ngh = a.getNghData(idx, d, c);
                    if (ngh.isValid()) {
                        partial += ngh.getData();
                        count++;
                    }
                }
                b(idx, c) = a(idx, c) - count * partial;
            }
        };
    });
}

template <typename Grid>
void dump(const std::string& path, typename Grid::template Field<int64_t, 0>& f, Neon::index_3d dim)
{
    std::vector<int64_t> dense(size_t(dim.rMul()), 0);
    f.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) { dense[p.x + size_t(dim.x) * (p.y + size_t(dim.y) * p.z)] = v; });
    std::ofstream o(path, std::ios::binary);
    o.write(reinterpret_cast<const char*>(dense.data()), dense.size() * sizeof(int64_t));
}

template <typename Grid>
void run(const std::string& outdir, Neon::index_3d dim, int iters)
{
    Neon::Backend bk(std::vector<int>{0}, Neon::Runtime::stream);
    Grid          grid(bk, dim, [](const Neon::index_3d&) { return true; }, Neon::domain::Stencil::s7_Laplace_t());
    auto          X = grid.template newField<int64_t, 0>("X", 1, 0);
    auto          Y = grid.template newField<int64_t, 0>("Y", 1, 0);
    // IODomain::resetValuesToMasked, digit 3: z + y 1e3 + x 1e6 + c 1e9 + offset 1e10
    auto masked = [](Neon::index_3d p, int64_t offset) { return int64_t(p.z) + 1000LL * p.y + 1000000LL * p.x + offset * 10000000000LL; };
    X.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) { v = masked(p, 1); });
    Y.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) { v = masked(p, 2); });
    X.updateDeviceData(0);
    Y.updateDeviceData(0);
    // Container::run: Y = L(X); X = L(Y)
    laplace(X, Y).run(0);
    laplace(Y, X).run(0);
    X.updateHostData(0);
    Y.updateHostData(0);
    bk.sync(0);
    const std::string tag = outdir + "/" + grid.getImplementationName() + "_" + std::to_string(dim.x) + "x" + std::to_string(dim.y) +
                            "x" + std::to_string(dim.z);
    dump<Grid>(tag + "_run_X.bin", X, dim);
    dump<Grid>(tag + "_run_Y.bin", Y, dim);

    // Skeleton: the same pair `iters` times from fresh values
    X.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) { v = masked(p, 1); });
    X.updateDeviceData(0);
    Neon::skeleton::Skeleton skl(bk);
    skl.sequence({laplace(X, Y), laplace(Y, X)}, "laplace");
    for (int i = 0; i < iters; i++) skl.run();
    X.updateHostData(0);
    bk.sync(0);
    dump<Grid>(tag + "_skel_X.bin", X, dim);

    // Neon's rule: a non-const field cannot be loaded for a STENCIL pattern
    bool threw = false;
    try {
        grid.newContainer("bad", [&](Neon::set::Loader& loader) {
                auto a = loader.load(X, Neon::Pattern::STENCIL);
                return [=] NEON_CUDA_HOST_DEVICE(const typename Grid::Idx&) mutable { (void)a; };
            })
            .run(0);
    } catch (const Neon::NeonException&) {
        threw = true;
    }
    std::printf("%s %dx%dx%d ok stencil-throw=%d\n", grid.getImplementationName().c_str(), dim.x, dim.y, dim.z, int(threw));
}

// eGrid on a sparse domain (cells with (x + y + z) % 3 != 0 active): inactive
// cells are not neighbours. Writes <grid>_<dims>_sparse_Y.bin (dense, 0 off the domain).
void run_sparse_egrid(const std::string& outdir, Neon::index_3d dim)
{
    Neon::Backend bk(std::vector<int>{0}, Neon::Runtime::stream);
    Neon::eGrid   grid(bk, dim, [](const Neon::index_3d& p) { return (p.x + p.y + p.z) % 3 != 0; },
                       Neon::domain::Stencil::s7_Laplace_t());
    auto          X = grid.newField<int64_t, 0>("X", 1, 0);
    auto          Y = grid.newField<int64_t, 0>("Y", 1, 0);
    X.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) {
        v = int64_t(p.z) + 1000LL * p.y + 1000000LL * p.x + 10000000000LL;
    });
    X.updateDeviceData(0);
    laplace(X, Y).run(0);
    Y.updateHostData(0);
    bk.sync(0);
    dump<Neon::eGrid>(outdir + "/eGrid_" + std::to_string(dim.x) + "x" + std::to_string(dim.y) + "x" + std::to_string(dim.z) +
                          "_sparse_Y.bin",
                      Y, dim);
    std::printf("eGrid sparse %dx%dx%d elements=%lld\n", dim.x, dim.y, dim.z, (long long)grid.getNumActiveCells());
}

int main(int argc, char** argv)
{
    const std::string outdir = argc > 1 ? argv[1] : ".";
    const int         iters = 5;
    // runHelper.h:36 dimensions; bGrid pads z to 24 for its tests (runHelper.h:77-81)
    for (auto d : {Neon::index_3d(10, 17, 13), Neon::index_3d(1, 1, 100), Neon::index_3d(17, 1, 77)}) {
        run<Neon::dGrid>(outdir, d, iters);
        run<Neon::eGrid>(outdir, d, iters);
        Neon::index_3d db = d;
        if (db.z < 24) db.z = 24;
        run<Neon::bGrid>(outdir, db, iters);
    }
    run_sparse_egrid(outdir, Neon::index_3d(19, 11, 23));
    return 0;
}
