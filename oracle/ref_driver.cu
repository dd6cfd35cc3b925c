// ORACLE — test infrastructure only.
//
// Harness around the reference's own D3Q19 lid-driven cavity, compiled from
// the reference's sources by oracle/ref_build.py into oracle/_ref/ and run on
// the reference's CPU backend (Neon::Runtime::openmp). It pins the oracle's
// restatement to outputs of the reference itself; nothing in the product
// library links or calls it.
//
// The set-up follows benchmarks/lbm-lid-driven-cavity-flow/src/RunCavityTwoPop.cu:19-242
// (backend, lattice, dGrid, the two population fields, the CellType field,
// LbmIterationD3Q19, the equilibrium / wall initialisation, the halo update
// and computeWallNghMask) and the time loop of :257-273; ν and ω come from the
// reference's own Config::parseArgs (Config.cpp:57-111). The harness adds only
// the copy of the newest populations into a caller buffer.
#include <cstdio>
#include <exception>
#include <string>
#include <vector>

// same include order as RunCavityTwoPop.cu:1-10 (CellType.h relies on the Neon headers before it)
#include "Config.h"
#include "D3Q19.h"
#include "Neon/domain/dGrid.h"

#include "CellType.h"
#include "LbmIteration.h"
#include "Neon/Neon.h"

namespace {

template <typename StorageFP, typename ComputeFP>
int run_cavity(int n, int steps, double ulb, double re, double* out, double* omega_out)
{
    using Lattice = D3Q19Template<StorageFP, ComputeFP>;
    using Grid = Neon::dGrid;
    using PopulationField = typename Grid::template Field<StorageFP, Lattice::Q>;

    Config config;
    config.Re = re;
    config.ulb = ulb;
    std::vector<std::string> args = {"ref_cavity",    "--deviceType", "cpu",
                                     "--deviceIds",   "0",            "--domain-size",
                                     std::to_string(n), "--computeFP", sizeof(ComputeFP) == 8 ? "double" : "float",
                                     "--storageFP",   sizeof(StorageFP) == 8 ? "double" : "float",
                                     "--benchmark"};
    std::vector<char*> argv;
    for (auto& a : args) argv.push_back(a.data());
    if (config.parseArgs(int(argv.size()), argv.data()) != 0) return -2;

    Neon::Backend bk(config.devices, Neon::Runtime::openmp);
    Neon::double_3d ulid(1., 0., 0.);
    Lattice         lattice(bk);
    Grid            grid(
        bk, {config.N, config.N, config.N}, [](const Neon::index_3d&) { return true; }, lattice.c_vect);
    PopulationField pop0 = grid.template newField<StorageFP, Lattice::Q>("Population", Lattice::Q, StorageFP(0.0));
    PopulationField pop1 = grid.template newField<StorageFP, Lattice::Q>("Population", Lattice::Q, StorageFP(0.0));
    CellType        defaultCelltype;
    auto            flag = grid.template newField<CellType, 1>("Material", 1, defaultCelltype);
    auto            lbmParameters = config.getLbmParameters<ComputeFP>();
    if (omega_out) *omega_out = double(lbmParameters.omega);

    LbmIterationD3Q19<PopulationField, ComputeFP> iteration(config.stencilSemantic, config.occ, config.transferMode, pop0, pop1,
                                                            flag, lbmParameters.omega);
    const Neon::index_3d dim(config.N, config.N, config.N);
    const auto&          t = lattice.t_vect;
    const auto&          c = lattice.c_vect;
    auto                 init = [&](const Neon::index_3d& idx, const int& k, StorageFP& val) {
        val = t.at(k);
        if (idx.x == 0 || idx.x == dim.x - 1 || idx.y == 0 || idx.y == dim.y - 1 || idx.z == 0 || idx.z == dim.z - 1) {
            if (idx.y == dim.y - 1)
                val = -6. * t.at(k) * config.ulb * (c.at(k).v[0] * ulid.v[0] + c.at(k).v[1] * ulid.v[1] + c.at(k).v[2] * ulid.v[2]);
            else
                val = 0;
        }
    };
    iteration.getInput().forEachActiveCell(init);
    iteration.getOutput().forEachActiveCell(init);
    flag.forEachActiveCell([&](const Neon::index_3d& idx, const int&, CellType& f) {
        f.classification = CellType::bulk;
        f.wallNghBitflag = 0;
        if (idx.x == 0 || idx.x == dim.x - 1 || idx.y == 0 || idx.y == dim.y - 1 || idx.z == 0 || idx.z == dim.z - 1) {
            f.classification = CellType::bounceBack;
            if (idx.y == dim.y - 1) f.classification = CellType::movingWall;
        }
    });
    iteration.getInput().updateDeviceData(Neon::Backend::mainStreamIdx);
    iteration.getOutput().updateDeviceData(Neon::Backend::mainStreamIdx);
    flag.updateDeviceData(Neon::Backend::mainStreamIdx);
    bk.syncAll();
    flag.newHaloUpdate(Neon::set::StencilSemantic::standard, Neon::set::TransferMode::get, Neon::Execution::device)
        .run(Neon::Backend::mainStreamIdx);
    bk.syncAll();
    LbmContainers<Lattice, PopulationField, ComputeFP>::computeWallNghMask(flag, flag).run(Neon::Backend::mainStreamIdx);
    bk.syncAll();

    for (int s = 0; s < steps; s++) iteration.run();
    bk.syncAll();

    auto& f = iteration.getInput();
    f.updateHostData(Neon::Backend::mainStreamIdx);
    bk.syncAll();
    const size_t V = size_t(n) * n * n;
    f.forEachActiveCell(
        [&](const Neon::index_3d& idx, const int& k, StorageFP& val) {
            out[size_t(k) * V + size_t(idx.x) + size_t(n) * (size_t(idx.y) + size_t(n) * size_t(idx.z))] = double(val);
        },
        Neon::computeMode_t::computeMode_e::seq);
    return 0;
}

bool g_init = false;

}  // namespace

extern "C" {

// D3Q19 BGK lid-driven cavity n^3 (lid u_lb along +x on y = n-1, Reynolds
// number re, equilibrium start), `steps` iterations of the reference's
// LbmIterationD3Q19 on its CPU backend. precision: 0 = FP64 storage and
// compute, 1 = FP32 storage and compute. out: 19 n^3 doubles, element
// (x, y, z, q) at x + n (y + n z) + q n^3 (the field layout of a single-device
// dGrid). *omega_out: the reference's omega. Returns 0, or < 0 on an exception.
int ref_cavity_run(int n, int steps, int precision, double ulb, double re, double* out, double* omega_out)
{
    try {
        if (!g_init) {
            Neon::init();
            g_init = true;
        }
        if (precision == 0) return run_cavity<double, double>(n, steps, ulb, re, out, omega_out);
        if (precision == 1) return run_cavity<float, float>(n, steps, ulb, re, out, omega_out);
        return -1;
    } catch (std::exception& e) {
        std::fprintf(stderr, "ref_cavity_run: %s\n", e.what());
        return -3;
    } catch (...) {
        std::fprintf(stderr, "ref_cavity_run: exception\n");
        return -3;
    }
}

}  // extern "C"
