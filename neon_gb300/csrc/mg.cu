// Grid-transfer and smoothing kernels of the multilevel learned
// preconditioner (FP32 fields, zero Dirichlet values on the box faces, the
// 7-point operator of ngb_laplacian_apply with spacing h).
//
// Levels are vertex-centred: coarse node I sits on fine node 2I, so a fine
// grid of n nodes per axis (n even) has a coarse grid of n/2 nodes with
// spacing 2h. The box-face nodes of every level are Fixed (value 0); the
// fine nodes n-2 (even) fall on the coarse face node n/2-1 and get no coarse
// correction there, which the smoothing on the fine level takes over.
//
//   restriction (full weighting, R = P^T / 8): rc(I) = sum_a w_a res(2I + a),
//       w = (1/4, 1/2, 1/4) per axis, on coarse interior nodes, 0 on faces;
//   prolongation (trilinear): u(i) += ec(i/2) for even i,
//       (ec((i-1)/2) + ec((i+1)/2)) / 2 for odd i, per axis, on fine Free nodes;
//   damped Jacobi: u' = u + omega h^2/6 (r - A u) on Free nodes, 0 on faces;
//       from u = 0 two sweeps are one stencil pass over r:
//       u2 = 2 c r - c^2 A r with c = omega h^2 / 6;
//   residual: res = r - A u on Free nodes, 0 on faces.
//
// The stencil passes walk 32 x 32 column tiles in z (mg_tile_kernel); restriction takes
// one thread per coarse node, prolongation one per fine x-pair.
#include <mutex>

#include "common.cuh"

namespace ngb {
namespace {

constexpr int kMgBX = 128;

struct Box {
    int32_t nx, ny, nz;
    float   inv_h2;  // 1 / h^2
};

__device__ __forceinline__ bool interior(const Box& b, int x, int y, int z)
{
    return x > 0 && y > 0 && z > 0 && x < b.nx - 1 && y < b.ny - 1 && z < b.nz - 1;
}

// Stencil passes on 32 x 32 column tiles: a CTA of 256 threads owns one
// tile (four cells per thread, rows ly0 + 8k) and walks a chunk of planes in
// z. Each plane of v goes through a double-buffered shared tile with a
// one-cell halo (one barrier per plane), the x and y neighbours come from
// there, the z neighbours and r from registers loaded one plane ahead.
// Offsets are 32-bit, relative to the chunk's first plane.
//   MODE 0: out = v + c (r - A v)        (one Jacobi sweep on u = v)
//   MODE 1: out = 2 c v - c^2 A v        (two sweeps from zero, v = r)
//   MODE 2: out = r - A v                (residual)
//   MODE 3: out = v                      (residual with u = 0, v = r)
//   MODE 4: out = A v
// Every mode writes 0 on the face nodes.
constexpr int kTileR = 4, kTileX = 32, kTileY = 8 * kTileR, kTileHalo = 2 * (kTileX + 2) + 2 * kTileY, kTileThreads = 256;
static_assert(kTileHalo <= kTileThreads, "one halo cell per thread at most");
constexpr int kMaxChunk = 32;

// planes per CTA: 32, halved (to 8 at least) until there are four CTAs per SM
int tile_chunk(const Box& b)
{
    static int            sms = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    });
    const int64_t tiles = int64_t((b.nx + kTileX - 1) / kTileX) * ((b.ny + kTileY - 1) / kTileY);
    int           zc = kMaxChunk;
    while (zc > 8 && tiles * ((b.nz + zc - 1) / zc) < int64_t(4) * sms) zc /= 2;
    return zc;
}

// the modes that read r keep 64 registers (four CTAs per SM), the others run at three
template <int MODE>
constexpr int tile_min_ctas()
{
    return (MODE == 0 || MODE == 2) ? 4 : 3;
}

template <int MODE>
__global__ void __launch_bounds__(kTileThreads, tile_min_ctas<MODE>())
    mg_tile_kernel(Box b, const float* __restrict__ v, const float* __restrict__ r, float* __restrict__ out, float c, int zc)
{
    constexpr int    R = kTileR, TY = kTileY;
    constexpr bool   kR = MODE == 0 || MODE == 2;
    __shared__ float planes[2][TY + 2][kTileX + 2];
    const int        lx = threadIdx.x % kTileX, ly0 = threadIdx.x / kTileX;
    // this thread's halo cell (threads < kTileHalo): the rows above and below, then the two side columns
    int        hx = 0, hy = 0;
    const bool halo = threadIdx.x < kTileHalo;
    if (threadIdx.x < kTileX + 2) {
        hx = threadIdx.x - 1, hy = -1;
    } else if (threadIdx.x < 2 * (kTileX + 2)) {
        hx = threadIdx.x - (kTileX + 2) - 1, hy = TY;
    } else if (halo) {
        const int k = threadIdx.x - 2 * (kTileX + 2);
        hx = (k & 1) ? kTileX : -1, hy = k >> 1;
    }
    const int     pl = b.nx * b.ny;
    const int     x = blockIdx.x * kTileX + lx, z0 = blockIdx.z * zc, z1 = min(z0 + zc, b.nz);
    const int64_t base = int64_t(z0) * pl;  // offsets below are relative to plane z0
    v += base;
    out += base;
    if (kR) r += base;
    bool own[R], in[R];
    int  stc[R], ix[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        const int y = blockIdx.y * TY + ly0 + 8 * k;
        own[k] = x < b.nx && y < b.ny;
        in[k] = own[k] && x > 0 && y > 0 && x < b.nx - 1 && y < b.ny - 1;
        stc[k] = own[k] ? pl : 0;  // cells outside the grid stay parked on offset 0 (read, never used or written)
        ix[k] = own[k] ? x + b.nx * y : 0;
    }
    const int  gx = blockIdx.x * kTileX + hx, gy = blockIdx.y * TY + hy;
    const bool hown = halo && gx >= 0 && gy >= 0 && gx < b.nx && gy < b.ny;
    const int  sth = hown ? pl : 0;
    int        ih = hown ? gx + b.nx * gy : 0;
    float      vm[R], vc[R], v1[R], r0[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        vm[k] = (own[k] && z0 >= 1) ? v[ix[k] - stc[k]] : 0.f;
        vc[k] = own[k] ? v[ix[k]] : 0.f;
        v1[k] = (own[k] && z0 + 1 < b.nz) ? v[ix[k] + stc[k]] : 0.f;
        r0[k] = (kR && own[k]) ? r[ix[k]] : 0.f;
    }
    float hv = hown ? v[ih] : 0.f;
    for (int z = z0; z < z1; z++) {
        // one plane of lookahead: these loads are used in the next iteration
        float v2[R], r1[R], hv1 = 0.f;
#pragma unroll
        for (int k = 0; k < R; k++) {
            v2[k] = (own[k] && z + 2 < b.nz) ? v[ix[k] + 2 * stc[k]] : 0.f;
            r1[k] = (kR && own[k] && z + 1 < z1) ? r[ix[k] + stc[k]] : 0.f;
        }
        if (hown && z + 1 < z1) hv1 = v[ih + sth];
        // buffer z & 1 was last read in iteration z - 2, before the barrier of iteration z - 1
        float (*plane)[kTileX + 2] = planes[z & 1];
#pragma unroll
        for (int k = 0; k < R; k++) plane[ly0 + 8 * k + 1][lx + 1] = vc[k];
        if (halo) plane[hy + 1][hx + 1] = hv;
        __syncthreads();
        const bool zin = z > 0 && z < b.nz - 1;
#pragma unroll
        for (int k = 0; k < R; k++) {
            const int ly = ly0 + 8 * k;
            float     o = 0.f;
            if (in[k] && zin) {
                if (MODE == 3) {
                    o = vc[k];
                } else {
                    const float left = plane[ly + 1][lx], right = plane[ly + 1][lx + 2];
                    const float dn = plane[ly][lx + 1], up = plane[ly + 2][lx + 1];
                    const float s = ((left + right) + (dn + up)) + (vm[k] + v1[k]);
                    const float av = __fmul_rn(__fmaf_rn(6.f, vc[k], -s), b.inv_h2);
                    if (MODE == 0) o = __fmaf_rn(c, r0[k] - av, vc[k]);
                    if (MODE == 1) o = __fmaf_rn(-c * c, av, 2.f * c * vc[k]);
                    if (MODE == 2) o = r0[k] - av;
                    if (MODE == 4) o = av;
                }
            }
            if (own[k]) out[ix[k]] = o;
            ix[k] += stc[k];
            vm[k] = vc[k], vc[k] = v1[k], v1[k] = v2[k], r0[k] = r1[k];
        }
        ih += sth;
        hv = hv1;
    }
}

template <int MODE>
int launch_tile(const Box& b, const float* v, const float* r, float* out, float c, cudaStream_t s)
{
    const int zc = tile_chunk(b);
    // 32-bit offsets within a chunk: (zc + 2) planes of nx * ny cells
    if (int64_t(b.nx) * b.ny * (zc + 2) >= (int64_t(1) << 31)) {
        set_error("multilevel kernels take planes of fewer than 2^31 / %d cells (nx * ny = %lld)", zc + 2, (long long)b.nx * b.ny);
        return NGB_ERR_RANGE;
    }
    const dim3 grid((b.nx + kTileX - 1) / kTileX, (b.ny + kTileY - 1) / kTileY, (b.nz + zc - 1) / zc);
    mg_tile_kernel<MODE><<<grid, kTileThreads, 0, s>>>(b, v, r, out, c, zc);
    NGB_LAUNCH_CHECK("mg_tile_kernel");
    return NGB_OK;
}

__global__ void __launch_bounds__(kMgBX) mg_restrict_kernel(Box f, Box c, const float* __restrict__ res, float* __restrict__ rc,
                                                           float scale)
{
    const int X = blockIdx.x * kMgBX + threadIdx.x, Y = blockIdx.y, Z = blockIdx.z;
    if (X >= c.nx) return;
    const int64_t o = X + int64_t(c.nx) * (Y + int64_t(c.ny) * Z);
    if (!interior(c, X, Y, Z)) {
        rc[o] = 0.f;
        return;
    }
    const int64_t sy = f.nx, sz = int64_t(f.nx) * f.ny;
    const int64_t i0 = 2 * X + sy * (2 * Y) + sz * (2 * Z);
    float         acc = 0.f;
#pragma unroll
    for (int dz = -1; dz <= 1; dz++) {
        float pz = 0.f;
#pragma unroll
        for (int dy = -1; dy <= 1; dy++) {
            const float* row = res + i0 + dz * sz + dy * sy;
            const float  px = 0.25f * (__ldg(row - 1) + __ldg(row + 1)) + 0.5f * __ldg(row);
            pz += (dy == 0 ? 0.5f : 0.25f) * px;
        }
        acc += (dz == 0 ? 0.5f : 0.25f) * pz;
    }
    rc[o] = scale * acc;
}

// One thread per fine x-pair (2X, 2X+1) of a row: fine 2X takes coarse X,
// fine 2X+1 the mean of X and X+1 (per axis likewise for y and z); the pair
// of u values is read and written as one float2.
__global__ void __launch_bounds__(kMgBX) mg_prolong_add_kernel(Box f, Box c, const float* __restrict__ ec, float* __restrict__ u)
{
    const int X = blockIdx.x * kMgBX + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (X >= c.nx || y == 0 || z == 0 || y == f.ny - 1 || z == f.nz - 1) return;
    const int64_t sy = c.nx, sz = int64_t(c.nx) * c.ny;
    const int     y0 = y >> 1, z0 = z >> 1;
    const bool    yo = y & 1, zo = z & 1;
    // sum over the coarse rows/planes of this fine (y, z) at coarse column Xc
    auto g = [&](int Xc) {
        const float* p = ec + Xc + sy * y0 + sz * z0;
        float        a = __ldg(p);
        if (yo) a += __ldg(p + sy);
        if (zo) {
            float t = __ldg(p + sz);
            if (yo) t += __ldg(p + sz + sy);
            a += t;
        }
        return a;
    };
    const float w = (yo ? 0.5f : 1.f) * (zo ? 0.5f : 1.f);
    const float g0 = g(X), g1 = X + 1 < c.nx ? g(X + 1) : 0.f;
    float2*     up = reinterpret_cast<float2*>(u + 2 * X + int64_t(f.nx) * (y + int64_t(f.ny) * z));
    float2      uv = *up;
    if (X > 0) uv.x += w * g0;                 // fine x = 2X (x = 0 is a face)
    if (2 * X + 1 < f.nx - 1) uv.y += 0.5f * w * (g0 + g1);  // fine x = 2X + 1 (x = nx - 1 is a face)
    *up = uv;
}

int check_desc(const ngb_poisson_desc* d)
{
    NGB_CHECK_ARG(d, "desc is NULL");
    NGB_CHECK_ARG(d->field == NGB_STORE_F32, "multilevel kernels take FP32 fields");
    NGB_CHECK_ARG(d->bd == nullptr, "multilevel kernels take the box-face Dirichlet problem (bd == NULL)");
    NGB_CHECK_ARG(d->nx >= 3 && d->ny >= 3 && d->nz >= 3, "dims must be at least 3");
    NGB_CHECK_ARG(d->ny <= 65535 && d->nz <= 65535, "ny and nz must be at most 65535");
    NGB_CHECK_ARG(d->h > 0, "h must be positive");
    return NGB_OK;
}

Box box_of(const ngb_poisson_desc* d) { return Box{d->nx, d->ny, d->nz, float(1.0 / (d->h * d->h))}; }

dim3 grid_of(const Box& b) { return dim3((b.nx + kMgBX - 1) / kMgBX, b.ny, b.nz); }

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_mg_jacobi(const ngb_poisson_desc* d, const void* u, const void* r, void* out, double omega, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(r && out && r != out && u != out, "r/out must be distinct non-NULL device pointers, u must differ from out");
    NGB_CHECK_ARG(omega > 0 && omega < 2, "omega must lie in (0, 2)");
    const Box   b = box_of(d);
    const float c = float(omega * d->h * d->h / 6.0);
    cudaStream_t s = as_stream(stream);
    if (u) return launch_tile<0>(b, static_cast<const float*>(u), static_cast<const float*>(r), static_cast<float*>(out), c, s);
    return launch_tile<1>(b, static_cast<const float*>(r), nullptr, static_cast<float*>(out), c, s);
}

int ngb_mg_residual(const ngb_poisson_desc* d, const void* u, const void* r, void* out, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(r && out && r != out && u != out, "r/out must be distinct non-NULL device pointers, u must differ from out");
    const Box    b = box_of(d);
    cudaStream_t s = as_stream(stream);
    if (u) return launch_tile<2>(b, static_cast<const float*>(u), static_cast<const float*>(r), static_cast<float*>(out), 0.f, s);
    return launch_tile<3>(b, static_cast<const float*>(r), nullptr, static_cast<float*>(out), 0.f, s);
}

int ngb_mg_apply(const ngb_poisson_desc* d, const void* u, void* out, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(u && out && u != out, "u/out must be distinct non-NULL device pointers");
    const Box b = box_of(d);
    return launch_tile<4>(b, static_cast<const float*>(u), nullptr, static_cast<float*>(out), 0.f, as_stream(stream));
}

int ngb_mg_restrict(const ngb_poisson_desc* fine, const void* res, void* rc_out, double scale, void* stream)
{
    int rc = check_desc(fine);
    if (rc) return rc;
    NGB_CHECK_ARG(fine->nx % 2 == 0 && fine->ny % 2 == 0 && fine->nz % 2 == 0 && fine->nx >= 6 && fine->ny >= 6 && fine->nz >= 6,
                  "fine dims must be even and at least 6");
    NGB_CHECK_ARG(res && rc_out && res != rc_out, "res/rc must be distinct non-NULL device pointers");
    const Box f = box_of(fine);
    const Box c{fine->nx / 2, fine->ny / 2, fine->nz / 2, f.inv_h2 * 0.25f};
    mg_restrict_kernel<<<grid_of(c), kMgBX, 0, as_stream(stream)>>>(f, c, static_cast<const float*>(res),
                                                                     static_cast<float*>(rc_out), float(scale));
    NGB_LAUNCH_CHECK("mg_restrict_kernel");
    return NGB_OK;
}

int ngb_mg_prolong_add(const ngb_poisson_desc* fine, const void* ec, void* u, void* stream)
{
    int rc = check_desc(fine);
    if (rc) return rc;
    NGB_CHECK_ARG(fine->nx % 2 == 0 && fine->ny % 2 == 0 && fine->nz % 2 == 0 && fine->nx >= 6 && fine->ny >= 6 && fine->nz >= 6,
                  "fine dims must be even and at least 6");
    NGB_CHECK_ARG(ec && u && ec != u, "ec/u must be distinct non-NULL device pointers");
    NGB_CHECK_ARG((reinterpret_cast<uintptr_t>(u) & 7) == 0, "u must be 8-byte aligned");
    const Box f = box_of(fine);
    const Box c{fine->nx / 2, fine->ny / 2, fine->nz / 2, f.inv_h2 * 0.25f};
    mg_prolong_add_kernel<<<dim3((c.nx + kMgBX - 1) / kMgBX, f.ny, f.nz), kMgBX, 0, as_stream(stream)>>>(
        f, c, static_cast<const float*>(ec), static_cast<float*>(u));
    NGB_LAUNCH_CHECK("mg_prolong_add_kernel");
    return NGB_OK;
}

}  // extern "C"
