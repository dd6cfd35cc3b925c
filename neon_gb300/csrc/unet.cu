// Kernels of the learned preconditioner (a small 3-D U-Net applied inside
// flexible CG): BF16 3x3x3 convolutions as implicit GEMMs on the tensor cores
// (mma m16n8k16, BF16 operands, FP32 accumulation), forward, backward-data
// and backward-weight, plus the pooling / upsampling / activation / optimiser
// glue. No reference counterpart (the reference has no learned solver).
//
// Tensors are channels-last on an nx*ny*nz grid: element (voxel v, channel c)
// at v*ld + c, v = x + nx*(y + ny*z); `ld` (row stride) lets a layer read or
// write a channel range of a wider buffer, which is how skip concatenations
// are formed without copies. Convolutions use zero padding.
#include "common.cuh"

#include <algorithm>
#include <cstdint>

namespace ngb {
namespace {

constexpr int kConvWarps = 4;   // warps per CTA
constexpr int kConvMT = 2;      // 16-row m tiles per warp (32 voxels)
constexpr int kMaxNT = 8;       // n tiles of 8 (Cout <= 64)

__device__ __forceinline__ uint32_t ld_b32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct Grid3 {
    int     nx, ny, nz;
    int64_t V;
};

// Linear neighbour index of voxel v at tap t (dz, dy, dx in {-1,0,1}, t = 9(dz+1)+3(dy+1)+(dx+1)), or -1.
__device__ __forceinline__ int64_t tap_ngh(const Grid3& g, int x, int y, int z, int t)
{
    const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
    const int X = x + dx, Y = y + dy, Z = z + dz;
    if (X < 0 || Y < 0 || Z < 0 || X >= g.nx || Y >= g.ny || Z >= g.nz) return -1;
    return X + int64_t(g.nx) * (Y + int64_t(g.ny) * Z);
}

// ---------------------------------------------------------------- convolution
// y[v][co] = act( sum_{t, ci} x[ngh(v,t)][ci] * w[co][t][ci] + bias[co] )
// OUT = __nv_bfloat16 (forward, optional ReLU) or float (backward data,
// optional accumulation into y). Cin % 16 == 0, Cout % 8 == 0, Cout <= 64.
template <typename OUT, int NT>
__global__ void __launch_bounds__(kConvWarps * 32) conv3d_kernel(Grid3 g, const __nv_bfloat16* __restrict__ x, int ldx, int cin,
                                                                 const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                                 OUT* __restrict__ y, int ldy, int relu, int accumulate)
{
    const int     lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int     gid = lane >> 2, tig = lane & 3;
    const int64_t v0 = (int64_t(blockIdx.x) * kConvWarps + warp) * (16 * kConvMT);
    // the 2*kConvMT voxels this thread loads A rows for
    int     vx[kConvMT][2], vy[kConvMT][2], vz[kConvMT][2];
    bool    vok[kConvMT][2];
#pragma unroll
    for (int m = 0; m < kConvMT; m++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int64_t v = v0 + m * 16 + gid + 8 * h;
            vok[m][h] = v < g.V;
            const int64_t vv = vok[m][h] ? v : 0;
            vx[m][h] = int(vv % g.nx);
            vy[m][h] = int((vv / g.nx) % g.ny);
            vz[m][h] = int(vv / (int64_t(g.nx) * g.ny));
        }
    float acc[kConvMT][NT][4];
#pragma unroll
    for (int m = 0; m < kConvMT; m++)
#pragma unroll
        for (int n = 0; n < NT; n++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[m][n][e] = 0.f;

    const int kpt = cin / 16;  // 16-channel chunks per tap
    const int K = 27 * cin;
    for (int t = 0; t < 27; t++) {
        int64_t src[kConvMT][2];
#pragma unroll
        for (int m = 0; m < kConvMT; m++)
#pragma unroll
            for (int h = 0; h < 2; h++) src[m][h] = vok[m][h] ? tap_ngh(g, vx[m][h], vy[m][h], vz[m][h], t) : -1;
        for (int kc = 0; kc < kpt; kc++) {
            const int c0 = kc * 16 + tig * 2;
            uint32_t  a[kConvMT][4];
#pragma unroll
            for (int m = 0; m < kConvMT; m++) {
                a[m][0] = src[m][0] >= 0 ? ld_b32(x + src[m][0] * ldx + c0) : 0u;
                a[m][1] = src[m][1] >= 0 ? ld_b32(x + src[m][1] * ldx + c0) : 0u;
                a[m][2] = src[m][0] >= 0 ? ld_b32(x + src[m][0] * ldx + c0 + 8) : 0u;
                a[m][3] = src[m][1] >= 0 ? ld_b32(x + src[m][1] * ldx + c0 + 8) : 0u;
            }
            const int kk = t * cin + kc * 16 + tig * 2;
#pragma unroll
            for (int n = 0; n < NT; n++) {
                const __nv_bfloat16* wr = w + int64_t(n * 8 + gid) * K + kk;
                const uint32_t       b[2] = {ld_b32(wr), ld_b32(wr + 8)};
#pragma unroll
                for (int m = 0; m < kConvMT; m++) mma_bf16(acc[m][n], a[m], b);
            }
        }
    }
    // epilogue: rows gid / gid+8, columns n*8 + 2 tig + {0,1}
#pragma unroll
    for (int m = 0; m < kConvMT; m++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (!vok[m][h]) continue;
            const int64_t v = v0 + m * 16 + gid + 8 * h;
#pragma unroll
            for (int n = 0; n < NT; n++) {
                const int co = n * 8 + tig * 2;
                float     r0 = acc[m][n][2 * h], r1 = acc[m][n][2 * h + 1];
                if (bias) r0 += bias[co], r1 += bias[co + 1];
                if constexpr (std::is_same<OUT, __nv_bfloat16>::value) {
                    if (relu) r0 = fmaxf(r0, 0.f), r1 = fmaxf(r1, 0.f);
                    *reinterpret_cast<__nv_bfloat162*>(y + v * ldy + co) = __floats2bfloat162_rn(r0, r1);
                } else {
                    float2* o = reinterpret_cast<float2*>(y + v * ldy + co);
                    if (accumulate) {
                        const float2 old = *o;
                        r0 += old.x, r1 += old.y;
                    }
                    *o = make_float2(r0, r1);
                }
            }
        }
}

// dw[co][t][ci] += sum_v dy[v][co] * x[ngh(v,t)][ci]: for one tap per blockIdx.y,
// a voxel chunk per blockIdx.x; M = Cout (m16 tiles), N = Cin (n8 tiles),
// K = voxels. Partial tiles go to dw with atomicAdd (FP32).
constexpr int kBwdChunk = 1024;  // voxels per CTA
template <int MT>
__global__ void __launch_bounds__(128) conv3d_bwd_weight_kernel(Grid3 g, const __nv_bfloat16* __restrict__ x, int ldx, int cin,
                                                                const __nv_bfloat16* __restrict__ dy, int lddy, int cout,
                                                                float* __restrict__ dw)
{
    const int     lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int     gid = lane >> 2, tig = lane & 3;
    const int     t = blockIdx.y;
    const int     ntiles = cin / 8;
    const int64_t vbeg = int64_t(blockIdx.x) * kBwdChunk;
    const int     K = 27 * cin;
    // each warp owns n tiles warp, warp+4, ... of Cin; all MT m tiles of Cout
    for (int nt = warp; nt < ntiles; nt += 4) {
        float acc[MT][4];
#pragma unroll
        for (int m = 0; m < MT; m++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[m][e] = 0.f;
        const int ci = nt * 8 + gid;
        for (int64_t k0 = vbeg; k0 < vbeg + kBwdChunk && k0 < g.V; k0 += 16) {
            // B (k = voxel, n = ci): rows 2 tig + {0,1} and +8
            uint32_t b[2];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                __nv_bfloat16 e2[2];
#pragma unroll
                for (int s = 0; s < 2; s++) {
                    const int64_t v = k0 + 8 * r + 2 * tig + s;
                    __nv_bfloat16 val = __float2bfloat16_rn(0.f);
                    if (v < g.V) {
                        const int     vx = int(v % g.nx), vy = int((v / g.nx) % g.ny), vz = int(v / (int64_t(g.nx) * g.ny));
                        const int64_t src = tap_ngh(g, vx, vy, vz, t);
                        if (src >= 0) val = x[src * ldx + ci];
                    }
                    e2[s] = val;
                }
                b[r] = uint32_t(__bfloat16_as_ushort(e2[0])) | (uint32_t(__bfloat16_as_ushort(e2[1])) << 16);
            }
#pragma unroll
            for (int m = 0; m < MT; m++) {
                // A (m = co, k = voxel): rows gid / gid+8, cols 2 tig + {0,1} and +8
                uint32_t a[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int     co = m * 16 + gid + 8 * (q & 1);
                    const int64_t v = k0 + 2 * tig + 8 * (q >> 1);
                    const __nv_bfloat16 lo = (v < g.V && co < cout) ? dy[v * lddy + co] : __float2bfloat16_rn(0.f);
                    const __nv_bfloat16 hi = (v + 1 < g.V && co < cout) ? dy[(v + 1) * lddy + co] : __float2bfloat16_rn(0.f);
                    a[q] = uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
                }
                mma_bf16(acc[m], a, b);
            }
        }
#pragma unroll
        for (int m = 0; m < MT; m++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int co = m * 16 + gid + 8 * (e >> 1);
                const int c = nt * 8 + 2 * tig + (e & 1);
                if (co < cout) atomicAdd(dw + int64_t(co) * K + t * cin + c, acc[m][e]);
            }
    }
}

// ---------------------------------------------------------------- elementwise glue
// out[v][c] = bf16(dy[v][c] * (y[v][c] > 0)) (ReLU backward; y may be NULL: no mask)
__global__ void relu_bwd_kernel(int64_t V, int C, const float* __restrict__ dy, int lddy, const __nv_bfloat16* __restrict__ y,
                                int ldy, __nv_bfloat16* __restrict__ out, int ldo)
{
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < V * C; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t v = i / C;
        const int     c = int(i % C);
        float         d = dy[v * lddy + c];
        if (y && !(__bfloat162float(y[v * ldy + c]) > 0.f)) d = 0.f;
        out[v * ldo + c] = __float2bfloat16_rn(d);
    }
}

// 2x2x2 average pooling (fine nx*ny*nz even) and its adjoint. The forward
// kernels walk coarse rows (Y, Z) with a block stride and a row's voxels
// (times channels) with a thread stride: one 32-bit division per row, and
// blocks that each move many rows (a block per row left the GPU scheduling
// blocks). Children summed in the order d = 0..7 (bit 0: x, bit 1: y, bit 2: z).
__global__ void pool2_kernel(Grid3 fine, int C, const __nv_bfloat16* __restrict__ x, int ldx, __nv_bfloat16* __restrict__ y, int ldy)
{
    const int cx = fine.nx / 2, cy = fine.ny / 2, rows = cy * (fine.nz / 2);
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const int Y = row % cy, Z = row / cy;
        for (int t = threadIdx.x; t < cx * C; t += blockDim.x) {
            const int     X = t / C, c = t - X * C;
            const int64_t vc = X + int64_t(cx) * (Y + int64_t(cy) * Z);
            float         s = 0.f;
#pragma unroll
            for (int d = 0; d < 8; d++) {
                const int64_t vf =
                    (2 * X + (d & 1)) + int64_t(fine.nx) * ((2 * Y + ((d >> 1) & 1)) + int64_t(fine.ny) * (2 * Z + (d >> 2)));
                s += __bfloat162float(x[vf * ldx + c]);
            }
            y[vc * ldy + c] = __float2bfloat16_rn(0.125f * s);
        }
    }
}
// The same with eight channels per thread (16-byte loads and stores): C, ldx
// and ldy multiples of 8, x and y 16-byte aligned.
__global__ void pool2_vec_kernel(Grid3 fine, int G, const uint4* __restrict__ x, int ldx8, uint4* __restrict__ y, int ldy8)
{
    const int cx = fine.nx / 2, cy = fine.ny / 2, rows = cy * (fine.nz / 2);
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const int Y = row % cy, Z = row / cy;
        for (int t = threadIdx.x; t < cx * G; t += blockDim.x) {
            const int     X = t / G, g = t - X * G;
            const int64_t vc = X + int64_t(cx) * (Y + int64_t(cy) * Z);
            float         s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int d = 0; d < 8; d++) {
                const int64_t vf =
                    (2 * X + (d & 1)) + int64_t(fine.nx) * ((2 * Y + ((d >> 1) & 1)) + int64_t(fine.ny) * (2 * Z + (d >> 2)));
                const uint4           w = __ldg(x + vf * ldx8 + g);
                const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&w);
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float2 f = __bfloat1622float2(h[e]);
                    s[2 * e] += f.x;
                    s[2 * e + 1] += f.y;
                }
            }
            uint4            o;
            __nv_bfloat162* oh = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
            for (int e = 0; e < 4; e++) oh[e] = __floats2bfloat162_rn(0.125f * s[2 * e], 0.125f * s[2 * e + 1]);
            y[vc * ldy8 + g] = o;
        }
    }
}
__global__ void pool2_bwd_kernel(Grid3 fine, int C, const float* __restrict__ dy, int lddy, float* __restrict__ dx, int lddx,
                                 int accumulate)
{
    const int cx = fine.nx / 2, cy = fine.ny / 2;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < fine.V * C; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t vf = i / C;
        const int     c = int(i % C);
        const int     x = int(vf % fine.nx), y = int((vf / fine.nx) % fine.ny), z = int(vf / (int64_t(fine.nx) * fine.ny));
        const int64_t vc = (x / 2) + int64_t(cx) * ((y / 2) + int64_t(cy) * (z / 2));
        const float   g = 0.125f * dy[vc * lddy + c];
        dx[vf * lddx + c] = accumulate ? dx[vf * lddx + c] + g : g;
    }
}
// Nearest 2x upsampling (coarse -> fine) and its adjoint (sum of the 8 children).
// Forward: fine rows (y, z) with a block stride, a row's voxels (times
// channels, or 8-channel groups) with a thread stride.
__global__ void up2_kernel(Grid3 fine, int C, const __nv_bfloat16* __restrict__ x, int ldx, __nv_bfloat16* __restrict__ y, int ldy)
{
    const int rows = fine.ny * fine.nz;
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const int yy = row % fine.ny, zz = row / fine.ny;
        for (int t = threadIdx.x; t < fine.nx * C; t += blockDim.x) {
            const int     xx = t / C, c = t - xx * C;
            const int64_t vf = xx + int64_t(fine.nx) * (yy + int64_t(fine.ny) * zz);
            const int64_t vc = (xx >> 1) + int64_t(fine.nx / 2) * ((yy >> 1) + int64_t(fine.ny / 2) * (zz >> 1));
            y[vf * ldy + c] = x[vc * ldx + c];
        }
    }
}
__global__ void up2_vec_kernel(Grid3 fine, int G, const uint4* __restrict__ x, int ldx8, uint4* __restrict__ y, int ldy8)
{
    const int rows = fine.ny * fine.nz;
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const int yy = row % fine.ny, zz = row / fine.ny;
        for (int t = threadIdx.x; t < fine.nx * G; t += blockDim.x) {
            const int     xx = t / G, g = t - xx * G;
            const int64_t vf = xx + int64_t(fine.nx) * (yy + int64_t(fine.ny) * zz);
            const int64_t vc = (xx >> 1) + int64_t(fine.nx / 2) * ((yy >> 1) + int64_t(fine.ny / 2) * (zz >> 1));
            y[vf * ldy8 + g] = __ldg(x + vc * ldx8 + g);
        }
    }
}
__global__ void up2_bwd_kernel(Grid3 fine, int C, const float* __restrict__ dy, int lddy, float* __restrict__ dx, int lddx)
{
    const int     cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
    const int64_t Vc = int64_t(cx) * cy * cz;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < Vc * C; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t vc = i / C;
        const int     c = int(i % C);
        const int     X = int(vc % cx), Y = int((vc / cx) % cy), Z = int(vc / (int64_t(cx) * cy));
        float         s = 0.f;
        for (int d = 0; d < 8; d++) {
            const int64_t vf = (2 * X + (d & 1)) + int64_t(fine.nx) * ((2 * Y + ((d >> 1) & 1)) + int64_t(fine.ny) * (2 * Z + (d >> 2)));
            s += dy[vf * lddy + c];
        }
        dx[vc * lddx + c] = s;
    }
}

// Adam on FP32 master weights; writes the BF16 copy used by the forward pass.
__global__ void adam_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ s,
                            float lr, float b1, float b2, float eps, float c1, float c2, __nv_bfloat16* __restrict__ pb)
{
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float si = b2 * s[i] + (1.f - b2) * gi * gi;
        m[i] = mi, s[i] = si;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(si / c2) + eps);
        p[i] = pi;
        if (pb) pb[i] = __float2bfloat16_rn(pi);
    }
}

// w[co][t][ci] (FP32 master) -> wt[ci][26 - t][co] (BF16): the weights of the
// backward-data convolution (transposed channels, mirrored taps).
__global__ void flip_weights_kernel(int cout, int cin, const float* __restrict__ w, __nv_bfloat16* __restrict__ wt)
{
    const int64_t n = int64_t(cout) * 27 * cin;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int co = int(i / (27 * cin));
        const int t = int((i / cin) % 27);
        const int ci = int(i % cin);
        wt[(int64_t(ci) * 27 + (26 - t)) * cout + co] = __float2bfloat16_rn(w[i]);
    }
}

int grid1d(int64_t n) { return int(std::min<int64_t>((n + 255) / 256, 152 * 16)); }

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

Grid3 make_grid(int nx, int ny, int nz) { return Grid3{nx, ny, nz, int64_t(nx) * ny * nz}; }

// Network input on the device: channel 0 of the channels-last BF16 input
// = bf16(r / sigma), sigma = sqrt(rr / V) (the field's RMS; 1 for a zero
// field). The network is bias-free with ReLU, so M(a r) = a M(r) for a > 0.
__global__ void unet_input_kernel(int64_t V, const float* __restrict__ r, const double* __restrict__ rr, __nv_bfloat16* in0,
                                  int32_t ld)
{
    const double ms = *rr / double(V);
    const float  sigma = ms > 0.0 ? float(sqrt(ms)) : 1.f;
    for (int64_t v = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < V; v += int64_t(gridDim.x) * blockDim.x)
        in0[v * ld] = __float2bfloat16_rn(r[v] / sigma);
}

// e = scale * sigma * out[:, 0] on interior nodes of the nx*ny*nz box, 0 on its faces.
__global__ void unet_output_kernel(int32_t nx, int32_t ny, int32_t nz, const float* __restrict__ out, int32_t ld,
                                   const double* __restrict__ rr, float scale, float* __restrict__ e)
{
    // rows (y, z) with a block stride, a row's voxels with a thread stride (no 64-bit division)
    const int64_t V = int64_t(nx) * ny * nz;
    const double  ms = *rr / double(V);
    const float   sigma = ms > 0.0 ? float(sqrt(ms)) : 1.f;
    const float   k = scale * sigma;
    for (int row = blockIdx.x; row < ny * nz; row += gridDim.x) {
        const int y = row % ny, z = row / ny;
        for (int x = threadIdx.x; x < nx; x += blockDim.x) {
            const int64_t v = x + int64_t(nx) * row;
            const bool    face = x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1;
            e[v] = face ? 0.f : out[v * ld] * k;
        }
    }
}

// e *= num / den when both are positive, else e = 0 (device scalars).
__global__ void scale_by_ratio_kernel(int64_t n, float* __restrict__ e, const double* __restrict__ num, const double* __restrict__ den)
{
    const double a = *num, b = *den;
    const float  beta = (a > 0.0 && b > 0.0) ? float(a / b) : 0.f;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) e[i] *= beta;
}

int stream_grid(int64_t n) { return int(std::min<int64_t>((n + 255) / 256, 152 * 16)); }

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_conv3d(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* w, const float* bias,
               void* y, int32_t ldy, int32_t cout, int32_t out_f32, int32_t relu, int32_t accumulate, void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "bad dims");
    NGB_CHECK_ARG(cin > 0 && cin % 16 == 0, "cin must be a positive multiple of 16 (got %d)", cin);
    NGB_CHECK_ARG(cout > 0 && cout % 8 == 0 && cout <= 64, "cout must be a multiple of 8 in [8, 64] (got %d)", cout);
    NGB_CHECK_ARG(ldx >= cin && ldy >= cout && ldx % 2 == 0 && ldy % 2 == 0, "bad leading dimensions");
    NGB_CHECK_ARG(x && w && y, "NULL argument");
    const Grid3  g = make_grid(nx, ny, nz);
    const int    vox_per_cta = kConvWarps * 16 * kConvMT;
    const int64_t blocks = (g.V + vox_per_cta - 1) / vox_per_cta;
    cudaStream_t s = as_stream(stream);
    const __nv_bfloat16* X = static_cast<const __nv_bfloat16*>(x);
    const __nv_bfloat16* W = static_cast<const __nv_bfloat16*>(w);
#define NGB_CONV(NT)                                                                                                       \
    if (out_f32)                                                                                                           \
        conv3d_kernel<float, NT><<<unsigned(blocks), kConvWarps * 32, 0, s>>>(g, X, ldx, cin, W, bias, static_cast<float*>(y), ldy, \
                                                                             relu, accumulate);                            \
    else                                                                                                                   \
        conv3d_kernel<__nv_bfloat16, NT><<<unsigned(blocks), kConvWarps * 32, 0, s>>>(                                    \
            g, X, ldx, cin, W, bias, static_cast<__nv_bfloat16*>(y), ldy, relu, accumulate);
    switch (cout / 8) {
        case 1: NGB_CONV(1) break;
        case 2: NGB_CONV(2) break;
        case 4: NGB_CONV(4) break;
        case 6: NGB_CONV(6) break;
        case 8: NGB_CONV(8) break;
        default: set_error("cout %d not instantiated (8, 16, 32, 48, 64)", cout); return NGB_ERR_UNSUPPORTED;
    }
#undef NGB_CONV
    NGB_LAUNCH_CHECK("conv3d_kernel");
    return NGB_OK;
}

int ngb_conv3d_bwd_weight(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* dy, int32_t lddy,
                          int32_t cout, float* dw, void* stream)
{
    if (ngb_conv3d_bwd_weight_tc_supported(nx, ny, nz, ldx, cin, lddy, cout) && (reinterpret_cast<uintptr_t>(x) & 15u) == 0 &&
        (reinterpret_cast<uintptr_t>(dy) & 15u) == 0 && dw)
        return ngb_conv3d_bwd_weight_tc(nx, ny, nz, x, ldx, cin, dy, lddy, cout, dw, stream);
    return ngb_conv3d_bwd_weight_mma(nx, ny, nz, x, ldx, cin, dy, lddy, cout, dw, stream);
}

int ngb_conv3d_bwd_weight_mma(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* dy,
                              int32_t lddy, int32_t cout, float* dw, void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "bad dims");
    NGB_CHECK_ARG(cin > 0 && cin % 16 == 0 && cout > 0 && cout <= 64 && cout % 8 == 0, "bad channel counts");
    NGB_CHECK_ARG(x && dy && dw, "NULL argument");
    const Grid3 g = make_grid(nx, ny, nz);
    const dim3  grid(unsigned((g.V + kBwdChunk - 1) / kBwdChunk), 27);
    cudaStream_t s = as_stream(stream);
    const __nv_bfloat16* X = static_cast<const __nv_bfloat16*>(x);
    const __nv_bfloat16* D = static_cast<const __nv_bfloat16*>(dy);
    switch ((cout + 15) / 16) {
        case 1: conv3d_bwd_weight_kernel<1><<<grid, 128, 0, s>>>(g, X, ldx, cin, D, lddy, cout, dw); break;
        case 2: conv3d_bwd_weight_kernel<2><<<grid, 128, 0, s>>>(g, X, ldx, cin, D, lddy, cout, dw); break;
        case 3: conv3d_bwd_weight_kernel<3><<<grid, 128, 0, s>>>(g, X, ldx, cin, D, lddy, cout, dw); break;
        default: conv3d_bwd_weight_kernel<4><<<grid, 128, 0, s>>>(g, X, ldx, cin, D, lddy, cout, dw); break;
    }
    NGB_LAUNCH_CHECK("conv3d_bwd_weight_kernel");
    return NGB_OK;
}

int ngb_relu_bwd(int64_t V, int32_t C, const float* dy, int32_t lddy, const void* y, int32_t ldy, void* out, int32_t ldo, void* stream)
{
    NGB_CHECK_ARG(V > 0 && C > 0 && dy && out, "bad argument");
    relu_bwd_kernel<<<grid1d(V * C), 256, 0, as_stream(stream)>>>(V, C, dy, lddy, static_cast<const __nv_bfloat16*>(y), ldy,
                                                                  static_cast<__nv_bfloat16*>(out), ldo);
    NGB_LAUNCH_CHECK("relu_bwd_kernel");
    return NGB_OK;
}

int ngb_pool2(int32_t nx, int32_t ny, int32_t nz, int32_t C, const void* x, int32_t ldx, void* y, int32_t ldy, void* stream)
{
    NGB_CHECK_ARG(nx % 2 == 0 && ny % 2 == 0 && nz % 2 == 0 && nx > 0 && C > 0 && x && y, "pool2 needs even dims");
    NGB_CHECK_ARG(int64_t(ny / 2) * (nz / 2) < (int64_t(1) << 31) && int64_t(nx / 2) * C < (int64_t(1) << 31), "pool2: grid too large");
    const int rows = std::min((ny / 2) * (nz / 2), 152 * 16);
    const Grid3 g = make_grid(nx, ny, nz);
    if (C % 8 == 0 && ldx % 8 == 0 && ldy % 8 == 0 && aligned16(x) && aligned16(y)) {
        const int G = C / 8;
        pool2_vec_kernel<<<rows, 256, 0, as_stream(stream)>>>(
            g, G, static_cast<const uint4*>(x), ldx / 8, static_cast<uint4*>(y), ldy / 8);
        NGB_LAUNCH_CHECK("pool2_vec_kernel");
    } else {
        pool2_kernel<<<rows, 256, 0, as_stream(stream)>>>(
            g, C, static_cast<const __nv_bfloat16*>(x), ldx, static_cast<__nv_bfloat16*>(y), ldy);
        NGB_LAUNCH_CHECK("pool2_kernel");
    }
    return NGB_OK;
}

int ngb_pool2_bwd(int32_t nx, int32_t ny, int32_t nz, int32_t C, const float* dy, int32_t lddy, float* dx, int32_t lddx,
                  int32_t accumulate, void* stream)
{
    NGB_CHECK_ARG(nx % 2 == 0 && ny % 2 == 0 && nz % 2 == 0 && nx > 0 && C > 0 && dy && dx, "pool2 needs even dims");
    const Grid3 g = make_grid(nx, ny, nz);
    pool2_bwd_kernel<<<grid1d(g.V * C), 256, 0, as_stream(stream)>>>(g, C, dy, lddy, dx, lddx, accumulate);
    NGB_LAUNCH_CHECK("pool2_bwd_kernel");
    return NGB_OK;
}

int ngb_up2(int32_t nx, int32_t ny, int32_t nz, int32_t C, const void* x, int32_t ldx, void* y, int32_t ldy, void* stream)
{
    NGB_CHECK_ARG(nx % 2 == 0 && ny % 2 == 0 && nz % 2 == 0 && nx > 0 && C > 0 && x && y, "up2 needs even fine dims");
    NGB_CHECK_ARG(int64_t(ny) * nz < (int64_t(1) << 31) && int64_t(nx) * C < (int64_t(1) << 31), "up2: grid too large");
    const int rows = int(std::min<int64_t>(int64_t(ny) * nz, 152 * 16));
    const Grid3 g = make_grid(nx, ny, nz);
    if (C % 8 == 0 && ldx % 8 == 0 && ldy % 8 == 0 && aligned16(x) && aligned16(y)) {
        const int G = C / 8;
        up2_vec_kernel<<<rows, 256, 0, as_stream(stream)>>>(g, G, static_cast<const uint4*>(x), ldx / 8, static_cast<uint4*>(y),
                                                              ldy / 8);
        NGB_LAUNCH_CHECK("up2_vec_kernel");
    } else {
        up2_kernel<<<rows, 256, 0, as_stream(stream)>>>(g, C, static_cast<const __nv_bfloat16*>(x), ldx,
                                                          static_cast<__nv_bfloat16*>(y), ldy);
        NGB_LAUNCH_CHECK("up2_kernel");
    }
    return NGB_OK;
}

int ngb_up2_bwd(int32_t nx, int32_t ny, int32_t nz, int32_t C, const float* dy, int32_t lddy, float* dx, int32_t lddx, void* stream)
{
    NGB_CHECK_ARG(nx % 2 == 0 && ny % 2 == 0 && nz % 2 == 0 && nx > 0 && C > 0 && dy && dx, "up2 needs even fine dims");
    const Grid3 g = make_grid(nx, ny, nz);
    up2_bwd_kernel<<<grid1d(g.V / 8 * C), 256, 0, as_stream(stream)>>>(g, C, dy, lddy, dx, lddx);
    NGB_LAUNCH_CHECK("up2_bwd_kernel");
    return NGB_OK;
}

int ngb_adam(int64_t n, float* p, const float* g, float* m, float* s, float lr, float b1, float b2, float eps, int32_t step, void* pb,
             void* stream)
{
    NGB_CHECK_ARG(n > 0 && p && g && m && s && step >= 1, "bad argument");
    const float c1 = 1.f - powf(b1, float(step)), c2 = 1.f - powf(b2, float(step));
    adam_kernel<<<grid1d(n), 256, 0, as_stream(stream)>>>(n, p, g, m, s, lr, b1, b2, eps, c1, c2, static_cast<__nv_bfloat16*>(pb));
    NGB_LAUNCH_CHECK("adam_kernel");
    return NGB_OK;
}

int ngb_flip_weights(int32_t cout, int32_t cin, const float* w, void* wt, void* stream)
{
    NGB_CHECK_ARG(cout > 0 && cin > 0 && w && wt, "bad argument");
    flip_weights_kernel<<<grid1d(int64_t(cout) * 27 * cin), 256, 0, as_stream(stream)>>>(cout, cin, w, static_cast<__nv_bfloat16*>(wt));
    NGB_LAUNCH_CHECK("flip_weights_kernel");
    return NGB_OK;
}

int ngb_unet_input(int64_t V, const float* r, const double* rr, void* in0, int32_t ld, void* stream)
{
    NGB_CHECK_ARG(V > 0 && ld >= 1, "V and ld must be positive");
    NGB_CHECK_ARG(r && rr && in0, "NULL pointer");
    unet_input_kernel<<<stream_grid(V), 256, 0, as_stream(stream)>>>(V, r, rr, static_cast<__nv_bfloat16*>(in0), ld);
    NGB_LAUNCH_CHECK("unet_input_kernel");
    return NGB_OK;
}

int ngb_unet_output(int32_t nx, int32_t ny, int32_t nz, const float* out, int32_t ld, const double* rr, double scale, float* e,
                    void* stream)
{
    NGB_CHECK_ARG(nx >= 1 && ny >= 1 && nz >= 1 && ld >= 1, "dims and ld must be positive");
    NGB_CHECK_ARG(out && rr && e, "NULL pointer");
    NGB_CHECK_ARG(int64_t(ny) * nz < (int64_t(1) << 31), "ny * nz must be below 2^31");
    unet_output_kernel<<<int(std::min<int64_t>(int64_t(ny) * nz, 152 * 16)), 256, 0, as_stream(stream)>>>(nx, ny, nz, out, ld, rr,
                                                                                                         float(scale), e);
    NGB_LAUNCH_CHECK("unet_output_kernel");
    return NGB_OK;
}

int ngb_scale_by_ratio(int64_t n, float* e, const double* num, const double* den, void* stream)
{
    NGB_CHECK_ARG(n > 0, "n must be positive");
    NGB_CHECK_ARG(e && num && den, "NULL pointer");
    scale_by_ratio_kernel<<<stream_grid(n), 256, 0, as_stream(stream)>>>(n, e, num, den);
    NGB_LAUNCH_CHECK("scale_by_ratio_kernel");
    return NGB_OK;
}

}  // extern "C"
