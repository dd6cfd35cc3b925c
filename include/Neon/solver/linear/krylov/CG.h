// CG_t<Grid, Real> (libNeonSolver/include/Neon/solver/linear/krylov/CG.h:70-76,
// src/linear/krylov/CG.cpp:14-183) over ngb_cg_solve.
//
// The iteration of CG.cpp:95-145 runs on the device: alpha, beta and the
// stopping decision never return to the host, the iteration is one CUDA
// graph, and the host polls a flag every 50 iterations. Differences from the
// reference, each deliberate: fields r, p, s in Real with FP64 reductions and
// an FP64 solution refreshed from the true residual every 50 iterations
// (iterative refinement); a Jacobi preconditioner (z = r / diag A); and the
// stopping test |b - A x| / |b| <= toleranceRel on the true residual (the
// reference compares delta = |r|^2 against sqrt(delta_0), CG.cpp:81,132).
#pragma once
#include <chrono>
#include <memory>

#include "Neon/solver/linear/IterativeLinearSolver.h"
#include "Neon/solver/linear/matvecs/LaplacianMatVec.h"

namespace Neon {
namespace solver {

#if defined(__CUDACC__)
template <typename A, typename B>
__global__ void ngb_cg_convert_kernel(int64_t n, const A* in, B* out)
{
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) out[i] = B(in[i]);
}
#endif

template <typename Grid, typename Real>
class CG_t {
   public:
    using Field = typename Grid::template Field<Real, 0>;
    using BdField = typename Grid::template Field<int8_t, 0>;
    using matVec_t = MatVec_t<Grid, Real>;

    auto name() const -> std::string { return "CG"; }
    void init(Field& x)
    {
        mBk = x.getBackend();
        mInit = true;
    }
    auto isInit() const -> bool { return mInit; }

#if defined(__CUDACC__)
    auto solve(std::shared_ptr<matVec_t> A, Field& x, Field& b, BdField& bd, const SolverParams& params,
               SolverResultInfo& result, const Neon::skeleton::Options& = Neon::skeleton::Options()) -> SolverStatus
    {
        if (!isInit()) {
            NeonException exc("CG_t::solve");
            exc << "Attempting to call solve() before calling init()";
            NEON_THROW(exc);
        }
        auto* lap = dynamic_cast<LaplacianMatVec<Grid, Real>*>(A.get());
        if (!lap) NEON_THROW_UNSUPPORTED_OPERATION("CG_t::solve runs the Laplacian operator (LaplacianMatVec)");
        const auto       t0 = std::chrono::steady_clock::now();
        const int32_3d   d = x.getDimension();
        const int64_t    n = int64_t(d.rMul());
        ngb_poisson_desc desc{d.x, d.y, d.z, sizeof(Real) == 8 ? NGB_STORE_F64 : NGB_STORE_F32, double(lap->stepSize()), bd.mem()};
        cudaStream_t     s = mBk.stream();
        const size_t     wsBytes = ngb_cg_workspace_bytes(&desc);
        if (wsBytes != mWsBytes) {
            if (mWs) cudaFree(mWs);
            if (mXh) cudaFree(mXh);
            NEON_CUDA_CHECK(cudaMalloc(&mWs, wsBytes));
            NEON_CUDA_CHECK(cudaMalloc(&mXh, size_t(n) * sizeof(double)));
            mWsBytes = wsBytes;
        }
        ngb_cg_convert_kernel<Real, double><<<256, 256, 0, s>>>(n, x.mem(), mXh);
        NEON_CUDA_CHECK(cudaGetLastError());
        ngb_cg_params prm{params.toleranceRel, int32_t(params.maxIterations), 50, 50, 1};
        ngb_cg_result res{};
        NEON_NGB_CHECK(ngb_cg_solve(&desc, b.mem(), mXh, mWs, mWsBytes, &prm, &res, s));
        ngb_cg_convert_kernel<double, Real><<<256, 256, 0, s>>>(n, mXh, x.mem());
        NEON_CUDA_CHECK(cudaGetLastError());
        NEON_CUDA_CHECK(cudaStreamSynchronize(s));
        result.solverName = name();
        result.numIterations = size_t(res.iterations);
        result.residualEnd = res.rel_residual;
        result.solveTime = res.seconds * 1e3;
        result.totalTime = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (res.converged) return SolverStatus::Converged;
        return res.iterations >= int32_t(params.maxIterations) ? SolverStatus::IterationLimit : SolverStatus::Error;
    }
#endif
    ~CG_t()
    {
        if (mWs) cudaFree(mWs);
        if (mXh) cudaFree(mXh);
    }

   private:
    Backend mBk;
    bool    mInit = false;
    void*   mWs = nullptr;
    double* mXh = nullptr;
    size_t  mWsBytes = 0;
};

}  // namespace solver
}  // namespace Neon
