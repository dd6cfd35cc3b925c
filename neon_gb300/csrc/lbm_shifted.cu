// Launches of the dense LBM kernels with FP32 compute (FP32 and 16-bit storage). Compiled with
// --fmad=false: the kernel writes every fused multiply-add explicitly.
#include "lbm_shifted.cuh"

namespace ngb {
namespace {

// Core kernel of the analytic cavity: the x-pair form for 16-bit D3Q19 when rows start on a word.
template <int Q, typename T>
void launch_core(bool pair, dim3 gpair, dim3 gcore, dim3 block, const T* fi, T* fo, const DenseParams<float>& ps,
                 const DirOffsets& o, cudaStream_t s)
{
    if constexpr (sizeof(T) == 2) {
        if (pair) {
            gpair.z = (gpair.z + PairWalk<T, Q>::planes - 1) / PairWalk<T, Q>::planes;
            lbm_box_core_pair_kernel<Q, T><<<gpair, kPairBlock, 0, s>>>(fi, fo, ps, o);
            return;
        }
    }
    lbm_box_core_kernel<Q, T><<<gcore, block, 0, s>>>(fi, fo, ps, o);
}

}  // namespace

int launch_lbm_dense_f32(int Q, int storage, const void* fin, void* fout, const uint32_t* flags, const DenseParams<float>& p,
                         cudaStream_t s)
{
    const dim3 grid((p.nx + kLbmBlockX - 1) / kLbmBlockX, p.ny, p.nz), block(kLbmBlockX);
    const int64_t esz = storage == NGB_STORE_F32 ? 4 : 2, sy = p.nx, sz = int64_t(p.nx) * p.ny;
    DirOffsets    o{};
    for (int q = 0; q < Q; q++) {
        const int cx = Q == 19 ? Lattice<19>::cx(q) : Lattice<27>::cx(q);
        const int cy = Q == 19 ? Lattice<19>::cy(q) : Lattice<27>::cy(q);
        const int cz = Q == 19 ? Lattice<19>::cz(q) : Lattice<27>::cz(q);
        o.own[q] = q * p.stride * esz;
        o.pull[q] = (q * p.stride - cx - cy * sy - cz * sz) * esz;
    }
    // FP16 values are 2^14 g: the wall terms added to them scale alike
    DenseParams<float> ps = p;
    if (storage == NGB_STORE_F16OFF || storage == NGB_STORE_F16SR)
        for (int c = 0; c < 2; c++)
            for (int q = 0; q < 27; q++) ps.wall[c][q] = p.wall[c][q] * NGB_F16OFF_SCALE;
    // Analytic cavity of at least 4 x 6 x 6 cells: core + shell kernels; otherwise one kernel over every
    // cell (D3Q27 with 16-bit storage and odd rows: the one-cell core measured slower than the one-kernel form).
    const bool split = lbm_dense_split(Q, storage, p);
    // 16-bit storage with even rows and planes: the x-pair core kernel (32-bit accesses)
    const bool pair = split && storage != NGB_STORE_F32 && p.nx % 2 == 0 && p.stride % 2 == 0;
    const dim3 gpair((p.nx / 2 + kPairBlock - 1) / kPairBlock, p.ny - 4, p.nz - 4);
    const dim3 gcore((p.nx - 1 + kLbmBlockX - 1) / kLbmBlockX, p.ny - 4, p.nz - 4);
    const dim3 gshell((p.nx - 1 + kLbmBlockX - 1) / kLbmBlockX, 2 * (p.ny - 2) + 2 * (p.nz - 4));
#define NGB_ONE(QQ, T)                                                                                                        \
    do {                                                                                                                      \
        const T* fi = static_cast<const T*>(fin);                                                                             \
        T*       fo = static_cast<T*>(fout);                                                                                  \
        if (split) {                                                                                                          \
            launch_core<QQ, T>(pair, gpair, gcore, block, fi, fo, ps, o, s);                                                  \
            lbm_box_shell_kernel<QQ, T><<<gshell, block, 0, s>>>(fi, fo, ps, o);                                              \
        } else {                                                                                                              \
            lbm_dense_single_kernel<QQ, T><<<grid, block, 0, s>>>(fi, fo, flags, ps, o);                                      \
        }                                                                                                                     \
    } while (0)
    const bool q19 = Q == 19;
    switch (storage) {
        case NGB_STORE_F32:
            if (q19) NGB_ONE(19, float); else NGB_ONE(27, float);
            break;
        case NGB_STORE_F16OFF:
            if (q19) NGB_ONE(19, __half); else NGB_ONE(27, __half);
            break;
        case NGB_STORE_F16SR:
            if (q19) NGB_ONE(19, f16sr_t); else NGB_ONE(27, f16sr_t);
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
