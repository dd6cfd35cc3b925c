// LaplacianMatVec<Grid, Real> (libNeonSolver/include/Neon/solver/linear/matvecs/LaplacianMatVec.h:17-59,
// src/linear/matvecs/LaplacianMatVec.cu:9-99) over ngb_laplacian_apply: Fixed rows
// copy the input, Free rows (n_valid u - sum of valid neighbours) / h^2.
#pragma once
#include <type_traits>

#include "Neon/domain/dGrid.h"
#include "Neon/solver/linear/IterativeLinearSolver.h"
#include "neon_gb300.h"

namespace Neon {
namespace solver {

template <typename Grid, typename Real>
class MatVec_t {
   public:
    using Field = typename Grid::template Field<Real, 0>;
    using bdField = typename Grid::template Field<int8_t, 0>;
    virtual ~MatVec_t() = default;
    virtual auto matVec(const Field& input, const bdField& boundary, Field& output) -> set::Container = 0;
};

template <typename Grid, typename Real>
class LaplacianMatVec : public MatVec_t<Grid, Real> {
   public:
    using Field = typename Grid::template Field<Real, 0>;
    using bdField = typename Grid::template Field<int8_t, 0>;
    static_assert(std::is_same_v<Grid, Neon::dGrid>, "the Laplacian operator runs on dGrid");
    static_assert(std::is_same_v<Real, float> || std::is_same_v<Real, double>, "Real must be float or double");

    explicit LaplacianMatVec(Real h) : m_h(h) {}
    auto stepSize() const -> Real { return m_h; }

    auto matVec(const Field& input, const bdField& boundary, Field& output) -> set::Container override
    {
        const double h = double(m_h);
        return set::Container("Laplacian", input.getBackend(), [input, boundary, output, h]() -> set::Launch {
            const int32_3d   d = input.getDimension();
            ngb_poisson_desc desc{d.x, d.y, d.z, std::is_same_v<Real, double> ? NGB_STORE_F64 : NGB_STORE_F32, h, boundary.mem()};
            set::Launch      l;
            l.signature = set::bytes_of(desc);
            const Real* in = input.mem();
            Real*       out = output.mem();
            l.signature.insert(l.signature.end(), reinterpret_cast<const char*>(&in), reinterpret_cast<const char*>(&in) + sizeof(in));
            l.run = [desc, in, out](cudaStream_t s) { NEON_NGB_CHECK(ngb_laplacian_apply(&desc, in, out, s)); };
            return l;
        });
    }

   private:
    Real m_h;
};

}  // namespace solver
}  // namespace Neon
