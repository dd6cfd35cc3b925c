// Data views and OCC on one partition, through the GB300 Neon API: the
// integer 6-neighbour operator of the domain-stencil test
// (libNeonDomain/tests/domain-stencil/src/stencil.cu:11-205) run
//   (1) over DataView::STANDARD,
//   (2) over DataView::INTERNAL only (dGrid: planes z = 1 .. nz - 2 written,
//       the two boundary planes untouched),
//   (3) then over DataView::BOUNDARY (every cell now equals (1)),
//   (4) in a Skeleton with Occ::standard (equal to (1)),
// and, for bGrid and eGrid, INTERNAL equal to STANDARD with BOUNDARY writing
// nothing (one partition: every block / element is internal).
// Prints one "dataview <grid> <dims> ok=<0|1>" line per case; exits 1 on any
// mismatch.
#include <cstdio>
#include <vector>

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
            const N              dirs[6] = {N(1, 0, 0), N(-1, 0, 0), N(0, 1, 0), N(0, -1, 0), N(0, 0, 1), N(0, 0, -1)};
            typename Field::Type partial = 0;
            int                  count = 0;
            for (const auto& d : dirs) {
                auto ngh = a.getNghData(idx, d, 0);
                if (ngh.isValid()) {
                    partial += ngh.getData();
                    count++;
                }
            }
            b(idx, 0) = a(idx, 0) - count * partial;
        };
    });
}

template <typename Field>
std::vector<int64_t> dense(Field& f, Neon::index_3d dim)
{
    std::vector<int64_t> d(size_t(dim.rMul()), -1);
    f.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) { d[p.x + size_t(dim.x) * (p.y + size_t(dim.y) * p.z)] = v; });
    return d;
}

template <typename Grid>
bool check(Neon::index_3d dim, bool dense_grid)
{
    constexpr int64_t kSentinel = -7;
    Neon::Backend     bk(std::vector<int>{0}, Neon::Runtime::stream);
    Grid              grid(bk, dim, [](const Neon::index_3d&) { return true; }, Neon::domain::Stencil::s7_Laplace_t());
    auto              X = grid.template newField<int64_t, 0>("X", 1, 0);
    auto              Y = grid.template newField<int64_t, 0>("Y", 1, 0);
    X.forEachActiveCell([&](const Neon::index_3d& p, int, int64_t& v) { v = int64_t(p.z) + 1000LL * p.y + 1000000LL * p.x + 1; });
    auto reset = [&]() {
        Y.forEachActiveCell([&](const Neon::index_3d&, int, int64_t& v) { v = kSentinel; });
        Y.updateDeviceData(0);
    };
    auto fetch = [&]() {
        Y.updateHostData(0);
        bk.sync(0);
        return dense(Y, dim);
    };
    X.updateDeviceData(0);
    reset();
    laplace(X, Y).run(0, Neon::DataView::STANDARD);
    const auto ref = fetch();

    bool ok = true;
    reset();
    laplace(X, Y).run(0, Neon::DataView::INTERNAL);
    const auto in = fetch();
    for (int z = 0; z < dim.z; z++)
        for (int y = 0; y < dim.y; y++)
            for (int x = 0; x < dim.x; x++) {
                const size_t i = x + size_t(dim.x) * (y + size_t(dim.y) * z);
                const bool   internal = !dense_grid || (z >= 1 && z < dim.z - 1);
                ok = ok && (internal ? in[i] == ref[i] : in[i] == kSentinel);
            }
    laplace(X, Y).run(0, Neon::DataView::BOUNDARY);
    ok = ok && fetch() == ref;

    reset();
    Neon::skeleton::Skeleton skl(bk);
    skl.sequence(std::vector<Neon::set::Container>{laplace(X, Y)}, "occ", Neon::skeleton::Options(Neon::skeleton::Occ::standard, Neon::set::TransferMode::get));
    skl.run();
    ok = ok && fetch() == ref;

    // the spans themselves: INTERNAL + BOUNDARY = STANDARD in cell count
    const auto s = grid.getSpan(Neon::Execution::device, 0, Neon::DataView::STANDARD);
    const auto si = grid.getSpan(Neon::Execution::device, 0, Neon::DataView::INTERNAL);
    const auto sb = grid.getSpan(Neon::Execution::device, 0, Neon::DataView::BOUNDARY);
    if constexpr (std::is_same_v<Grid, Neon::dGrid>) ok = ok && si.dim.z + sb.dim.z == s.dim.z;
    else if constexpr (std::is_same_v<Grid, Neon::bGrid>) ok = ok && si.nBlocks == s.nBlocks && sb.nBlocks == 0;
    else ok = ok && si.count == s.count && sb.count == 0;

    std::printf("dataview %s %dx%dx%d ok=%d\n", grid.getImplementationName().c_str(), dim.x, dim.y, dim.z, ok ? 1 : 0);
    return ok;
}

int main()
{
    Neon::init();
    bool ok = true;
    for (auto d : {Neon::index_3d(10, 17, 13), Neon::index_3d(17, 1, 77), Neon::index_3d(5, 6, 2), Neon::index_3d(4, 4, 1)})
        ok = check<Neon::dGrid>(d, true) && ok;
    for (auto d : {Neon::index_3d(10, 17, 24), Neon::index_3d(17, 1, 77)}) ok = check<Neon::bGrid>(d, false) && ok;
    for (auto d : {Neon::index_3d(10, 17, 13), Neon::index_3d(3, 1, 40)}) ok = check<Neon::eGrid>(d, false) && ok;
    return ok ? 0 : 1;
}
