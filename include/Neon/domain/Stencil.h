// Neon::domain::Stencil (libNeonDomain/src/domain/interface/Stencil.cpp:7-173):
// the list of neighbour offsets a grid serves.
#pragma once
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "Neon/core/core.h"

namespace Neon {
namespace domain {

class Stencil {
   public:
    Stencil() = default;
    Stencil(const std::vector<index_3d>& points, bool filterCenterOut = true)
    {
        for (const auto& p : points)
            if (!(filterCenterOut && p == index_3d(0, 0, 0))) mPoints.push_back(p);
    }
    auto neighbours() const -> const std::vector<index_3d>& { return mPoints; }
    auto nNeighbours() const -> int { return int(mPoints.size()); }
    auto nPoints() const -> int { return int(mPoints.size()); }
    auto getRadius() const -> int
    {
        int r = 0;
        for (auto& p : mPoints) r = std::max(r, std::max(std::abs(p.x), std::max(std::abs(p.y), std::abs(p.z))));
        return r;
    }
    static Stencil s7_Laplace_t() { return Stencil({{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}}); }
    static Stencil s27_t(bool filterCenterOut)
    {
        std::vector<index_3d> p;
        for (int x = -1; x <= 1; x++)
            for (int y = -1; y <= 1; y++)
                for (int z = -1; z <= 1; z++) p.push_back(index_3d(x, y, z));
        return Stencil(p, filterCenterOut);
    }
    static Stencil s19_t(bool filterCenterOut)
    {
        std::vector<index_3d> p;
        for (int x = -1; x <= 1; x++)
            for (int y = -1; y <= 1; y++)
                for (int z = -1; z <= 1; z++)
                    if (std::abs(x) + std::abs(y) + std::abs(z) <= 2) p.push_back(index_3d(x, y, z));
        return Stencil(p, filterCenterOut);
    }

   private:
    std::vector<index_3d> mPoints;
};

}  // namespace domain
}  // namespace Neon
