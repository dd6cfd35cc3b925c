// FP64 instantiations of the dense LBM step. This translation unit is compiled
// with --fmad=false so that the double-precision arithmetic keeps the
// operation order of the reference expressions (no fused multiply-adds).
#include "lbm_kernels.cuh"

namespace ngb {

int launch_lbm_dense_f64(int Q, const void* fin, void* fout, const uint32_t* flags, const DenseParams<double>& p, cudaStream_t s)
{
    const dim3 grid((p.nx + kLbmBlockX - 1) / kLbmBlockX, p.ny, p.nz), block(kLbmBlockX);
    if (Q == 19)
        lbm_dense_f64_kernel<19, double><<<grid, block, 0, s>>>(static_cast<const double*>(fin), static_cast<double*>(fout), flags, p);
    else
        lbm_dense_f64_kernel<27, double><<<grid, block, 0, s>>>(static_cast<const double*>(fin), static_cast<double*>(fout), flags, p);
    NGB_LAUNCH_CHECK("lbm_dense_f64_kernel");
    return NGB_OK;
}

}  // namespace ngb
