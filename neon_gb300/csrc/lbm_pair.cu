// Instantiations of the two-cells-per-thread dense LBM kernel. Compiled with
// --fmad=false: the kernel writes every fused multiply-add explicitly.
#include "lbm_pair.cuh"
#include <cstdlib>

namespace ngb {

// Returns NGB_ERR_UNSUPPORTED (without launching) when the pair layout does
// not apply: odd nx, odd plane stride or buffers not aligned to one pair.
int launch_lbm_dense_pair(int Q, int storage, const void* fin, void* fout, const uint32_t* flags, const DenseParams<float>& p,
                          cudaStream_t s)
{
    const size_t esz = storage == NGB_STORE_F32 ? 4 : 2;
    const size_t align = 2 * esz;
    if ((p.nx & 1) || (p.stride & 1) || (reinterpret_cast<uintptr_t>(fin) % align) || (reinterpret_cast<uintptr_t>(fout) % align))
        return NGB_ERR_UNSUPPORTED;
    const dim3 block(kPairX, kPairY);
    const dim3 grid((p.nx / 2 + kPairX - 1) / kPairX, (p.ny + kPairY - 1) / kPairY, p.nz);
#define NGB_PAIR(QQ, T) \
    lbm_dense_pair_kernel<QQ, T><<<grid, block, 0, s>>>(static_cast<const T*>(fin), static_cast<T*>(fout), flags, p)
    const bool q19 = Q == 19;
    switch (storage) {
        case NGB_STORE_F32:
            if (q19) NGB_PAIR(19, float); else NGB_PAIR(27, float);
            break;
        case NGB_STORE_F16OFF:
            if (q19) NGB_PAIR(19, __half); else NGB_PAIR(27, __half);
            break;
        case NGB_STORE_BF16OFF:
            if (q19) NGB_PAIR(19, __nv_bfloat16); else NGB_PAIR(27, __nv_bfloat16);
            break;
        default: return NGB_ERR_UNSUPPORTED;
    }
#undef NGB_PAIR
    NGB_LAUNCH_CHECK("lbm_dense_pair_kernel");
    return NGB_OK;
}

int launch_lbm_dense_f32(int Q, int storage, const void* fin, void* fout, const uint32_t* flags, const DenseParams<float>& p,
                         cudaStream_t s)
{
    // Kernel shape (all run the same IEEE operation sequence per cell):
    // NGB_LBM_VARIANT = 0 one cell per thread, 1 two cells along x, 2 two cells along z.
    static const int variant = [] {
        const char* e = getenv("NGB_LBM_VARIANT");
        return e ? atoi(e) : 0;
    }();
    if (variant == 1) {
        int rc = launch_lbm_dense_pair(Q, storage, fin, fout, flags, p, s);
        if (rc != NGB_ERR_UNSUPPORTED) return rc;
    }
    if (variant == 2) {
        const dim3 g2((p.nx + kLbmBlockX - 1) / kLbmBlockX, p.ny, (p.nz + 1) / 2), b2(kLbmBlockX);
#define NGB_ZP(QQ, T) \
    lbm_dense_zpair_kernel<QQ, T><<<g2, b2, 0, s>>>(static_cast<const T*>(fin), static_cast<T*>(fout), flags, p)
        const bool q19z = Q == 19;
        switch (storage) {
            case NGB_STORE_F32:
                if (q19z) NGB_ZP(19, float); else NGB_ZP(27, float);
                break;
            case NGB_STORE_F16OFF:
                if (q19z) NGB_ZP(19, __half); else NGB_ZP(27, __half);
                break;
            case NGB_STORE_BF16OFF:
                if (q19z) NGB_ZP(19, __nv_bfloat16); else NGB_ZP(27, __nv_bfloat16);
                break;
            default: set_error("unsupported storage %d", storage); return NGB_ERR_UNSUPPORTED;
        }
#undef NGB_ZP
        NGB_LAUNCH_CHECK("lbm_dense_zpair_kernel");
        return NGB_OK;
    }
    const dim3 grid((p.nx + kLbmBlockX - 1) / kLbmBlockX, p.ny, p.nz), block(kLbmBlockX);
#define NGB_ONE(QQ, T) \
    lbm_dense_single_kernel<QQ, T><<<grid, block, 0, s>>>(static_cast<const T*>(fin), static_cast<T*>(fout), flags, p)
    const bool q19 = Q == 19;
    switch (storage) {
        case NGB_STORE_F32:
            if (q19) NGB_ONE(19, float); else NGB_ONE(27, float);
            break;
        case NGB_STORE_F16OFF:
            if (q19) NGB_ONE(19, __half); else NGB_ONE(27, __half);
            break;
        case NGB_STORE_BF16OFF:
            if (q19) NGB_ONE(19, __nv_bfloat16); else NGB_ONE(27, __nv_bfloat16);
            break;
        default: set_error("unsupported storage %d", storage); return NGB_ERR_UNSUPPORTED;
    }
#undef NGB_ONE
    NGB_LAUNCH_CHECK("lbm_dense_single_kernel");
    return NGB_OK;
}

}  // namespace ngb
