// LearnedFCG_t<Grid, Real>: the learned-preconditioner sibling of CG_t
// (libNeonSolver/include/Neon/solver/linear/krylov/CG.h:70-76) over
// ngb_learned_solve, with CG_t's solve(A, x, b, bd, params, result) shape.
//
// Flexible CG preconditioned by a V-cycle whose coarsest-level solve is the
// U-Net (trained weights from a file written by ngb_unet_write_weights); the
// solution accumulates in FP64 and the true residual |b - A x| / |b| decides
// convergence; Jacobi-PCG takes over on stagnation. It solves the
// zero-Dirichlet box problem of LaplacianMatVec (every face Fixed, h = 1) on
// a cubic grid whose size is a multiple of 2^levels: other boundary
// layouts or spacings are rejected with NEON_THROW_UNSUPPORTED_OPERATION.
#pragma once
#include <chrono>
#include <memory>
#include <string>
#include <vector>

#include "Neon/solver/linear/krylov/CG.h"

namespace Neon {
namespace solver {

template <typename Grid, typename Real>
class LearnedFCG_t {
   public:
    using Field = typename Grid::template Field<Real, 0>;
    using BdField = typename Grid::template Field<int8_t, 0>;
    using matVec_t = MatVec_t<Grid, Real>;

    // weightsPath: a U-Net weight file; levels: V-cycle levels above the network's grid
    LearnedFCG_t(std::string weightsPath, int levels) : mPath(std::move(weightsPath)), mLevels(levels) {}
    LearnedFCG_t(const LearnedFCG_t&) = delete;
    LearnedFCG_t& operator=(const LearnedFCG_t&) = delete;

    auto name() const -> std::string { return "LearnedFCG"; }
    void init(Field& x)
    {
        mBk = x.getBackend();
        mInit = true;
    }
    auto isInit() const -> bool { return mInit; }

#if defined(__CUDACC__)
    auto solve(std::shared_ptr<matVec_t> A, Field& x, Field& b, BdField& /*bd*/, const SolverParams& params,
               SolverResultInfo& result, const Neon::skeleton::Options& = Neon::skeleton::Options()) -> SolverStatus
    {
        static_assert(sizeof(Real) == 4, "LearnedFCG_t takes FP32 fields (the solution accumulates in FP64 inside)");
        if (!isInit()) {
            NeonException exc("LearnedFCG_t::solve");
            exc << "Attempting to call solve() before calling init()";
            NEON_THROW(exc);
        }
        auto* lap = dynamic_cast<LaplacianMatVec<Grid, Real>*>(A.get());
        if (!lap || lap->stepSize() != Real(1))
            NEON_THROW_UNSUPPORTED_OPERATION("LearnedFCG_t::solve runs the unit-spacing Laplacian (LaplacianMatVec, h = 1)");
        const auto     t0 = std::chrono::steady_clock::now();
        const int32_3d d = x.getDimension();
        if (d.x != d.y || d.x != d.z) NEON_THROW_UNSUPPORTED_OPERATION("LearnedFCG_t::solve needs a cubic grid");
        const int64_t n = int64_t(d.rMul());
        if (!mSolver || mN != d.x) {
            release();
            std::vector<float> w(static_cast<size_t>(ngb_unet_weight_count()));
            NEON_NGB_CHECK(ngb_unet_read_weights(mPath.c_str(), w.data(), int64_t(w.size())));
            NEON_NGB_CHECK(ngb_learned_create(d.x, mLevels, w.data(), int64_t(w.size()), &mSolver));
            NEON_CUDA_CHECK(cudaMalloc(&mXh, size_t(n) * sizeof(double)));
            mN = d.x;
        }
        cudaStream_t s = mBk.stream();
        ngb_cg_convert_kernel<Real, double><<<256, 256, 0, s>>>(n, x.mem(), mXh);
        NEON_CUDA_CHECK(cudaGetLastError());
        ngb_learned_params prm{params.toleranceRel, int32_t(params.maxIterations), 10, 30, 1};
        ngb_learned_result res{};
        NEON_NGB_CHECK(ngb_learned_solve(mSolver, b.mem(), mXh, &prm, &res, s));
        ngb_cg_convert_kernel<double, Real><<<256, 256, 0, s>>>(n, mXh, x.mem());
        NEON_CUDA_CHECK(cudaGetLastError());
        NEON_CUDA_CHECK(cudaStreamSynchronize(s));
        result.solverName = name();
        result.numIterations = size_t(res.iterations) + size_t(res.fallback_iterations);
        result.residualEnd = res.rel_residual;
        result.solveTime = res.seconds * 1e3;
        result.totalTime = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        mFallback = res.fallback != 0;
        if (res.converged) return SolverStatus::Converged;
        return SolverStatus::IterationLimit;
    }
#endif
    // whether the last solve handed over to Jacobi-PCG
    auto usedFallback() const -> bool { return mFallback; }

    ~LearnedFCG_t() { release(); }

   private:
    void release()
    {
        if (mSolver) ngb_learned_destroy(mSolver);
        if (mXh) cudaFree(mXh);
        mSolver = nullptr;
        mXh = nullptr;
    }
    std::string         mPath;
    int                 mLevels;
    Backend             mBk;
    bool                mInit = false;
    bool                mFallback = false;
    ngb_learned_solver* mSolver = nullptr;
    double*             mXh = nullptr;
    int                 mN = 0;
};

}  // namespace solver
}  // namespace Neon
