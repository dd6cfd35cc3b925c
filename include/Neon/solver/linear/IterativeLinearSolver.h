// libNeonSolver's solver vocabulary (include/Neon/solver/linear/IterativeLinearSolver.h:17-33, 163-188).
#pragma once
#include <string>
#include <vector>

#include "Neon/core/core.h"
#include "Neon/skeleton/Skeleton.h"

namespace Neon {
namespace solver {

// Solvers use 0 for Dirichlet (Fixed) and 1 for Free degrees of freedom.
enum BoundaryCondition : int8_t { Fixed = 0, Free = 1 };

struct SolverParams {
    size_t                  maxIterations = 100;
    double                  toleranceRel = 1e-5;  // here: on the true residual |b - A x| / |b|
    double                  toleranceAbs = 0.0;
    double                  toleranceDiv = 1e+5;
    bool                    needResiduals = false;
    bool                    numericalIssueIsFailure = true;
    Neon::skeleton::Options skeletonOptions;
};

enum class SolverStatus { Converged, Iterating, IterationLimit, Error };

struct SolverResultInfo {
    std::string         solverName;
    size_t              numIterations = 0;
    double              residualStart = 0;
    double              residualEnd = 0;
    std::vector<double> residuals;
    double              solveTime = 0;  // ms
    double              totalTime = 0;  // ms
};

}  // namespace solver
}  // namespace Neon
