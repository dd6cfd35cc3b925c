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
// The stencil passes walk columns in z (mg_column_kernel); restriction takes
// one thread per coarse node, prolongation one per fine x-pair.
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

// Stencil passes as column walks: a CTA of 32 x 8 threads owns 32 x 8
// columns and walks kZChunk planes in z; the column's stencil values at
// z-1 .. z+4 and r at z .. z+3 stay in registers (a prefetch ring three
// planes deep), the x neighbours come from the adjacent lanes (shuffles; the
// two tile-edge lanes load theirs), the y neighbours from the rows the
// CTA's other warps loaded planes earlier (L1).
//   MODE 0: out = v + c (r - A v)        (one Jacobi sweep on u = v)
//   MODE 1: out = 2 c v - c^2 A v        (two sweeps from zero, v = r)
//   MODE 2: out = r - A v                (residual)
//   MODE 3: out = v                      (residual with u = 0, v = r)
//   MODE 4: out = A v
// Every mode writes 0 on the face nodes.
constexpr int kZX = 32, kZY = 8, kZChunk = 32;

template <int MODE>
__global__ void __launch_bounds__(kZX * kZY) mg_column_kernel(Box b, const float* __restrict__ v, const float* __restrict__ r,
                                                             float* __restrict__ out, float c)
{
    const int     lane = threadIdx.x;
    const int     x = blockIdx.x * kZX + lane, y = blockIdx.y * kZY + threadIdx.y;
    const int     z0 = blockIdx.z * kZChunk, z1 = min(z0 + kZChunk, b.nz);
    const bool    col = x < b.nx && y < b.ny;
    const bool    inner_col = col && x > 0 && y > 0 && x < b.nx - 1 && y < b.ny - 1;
    const int64_t sy = b.nx, sz = int64_t(b.nx) * b.ny;
    const int64_t i0 = col ? x + sy * y : 0;
    auto          at = [&](int zz) { return (col && zz >= 0 && zz < b.nz) ? __ldg(v + i0 + sz * zz) : 0.f; };
    constexpr bool kR = MODE == 0 || MODE == 2;
    auto          rat = [&](int zz) { return (kR && col && zz < b.nz) ? __ldg(r + i0 + sz * zz) : 0.f; };
    // the column's stencil values z-1 .. z+4 and r at z .. z+2 in registers: three planes of
    // loads stay in flight while a plane is computed (a load used in its own trip exposed the
    // whole DRAM latency once per plane)
    // (planes beyond the chunk's last stencil source z1 are not loaded)
    auto  atc = [&](int zz) { return zz <= z1 ? at(zz) : 0.f; };
    auto  ratc = [&](int zz) { return zz < z1 ? rat(zz) : 0.f; };
    float vm = at(z0 - 1), vc = at(z0), v1 = atc(z0 + 1), v2 = atc(z0 + 2), v3 = atc(z0 + 3);
    float r0 = ratc(z0), r1 = ratc(z0 + 1), r2 = ratc(z0 + 2);
    for (int z = z0; z < z1; z++) {
        const float   v4 = atc(z + 4);
        const float   r3 = ratc(z + 3);
        const float   vp = v1;
        float         left = __shfl_up_sync(0xffffffffu, vc, 1), right = __shfl_down_sync(0xffffffffu, vc, 1);
        const int64_t i = i0 + sz * z;
        if (lane == 0) left = (inner_col && z > 0 && z < b.nz - 1) ? __ldg(v + i - 1) : 0.f;
        if (lane == kZX - 1) right = (inner_col && z > 0 && z < b.nz - 1) ? __ldg(v + i + 1) : 0.f;
        if (col) {
            float o = 0.f;
            if (inner_col && z > 0 && z < b.nz - 1) {
                if (MODE == 3) {
                    o = vc;
                } else {
                    const float s = ((left + right) + (__ldg(v + i - sy) + __ldg(v + i + sy))) + (vm + vp);
                    const float av = __fmul_rn(__fmaf_rn(6.f, vc, -s), b.inv_h2);
                    if (MODE == 0) o = __fmaf_rn(c, r0 - av, vc);
                    if (MODE == 1) o = __fmaf_rn(-c * c, av, 2.f * c * vc);
                    if (MODE == 2) o = r0 - av;
                    if (MODE == 4) o = av;
                }
            }
            out[i] = o;
        }
        vm = vc;
        vc = v1;
        v1 = v2;
        v2 = v3;
        v3 = v4;
        r0 = r1;
        r1 = r2;
        r2 = r3;
    }
}

dim3 column_grid(const Box& b) { return dim3((b.nx + kZX - 1) / kZX, (b.ny + kZY - 1) / kZY, (b.nz + kZChunk - 1) / kZChunk); }

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
    const dim3 blk(kZX, kZY);
    if (u)
        mg_column_kernel<0><<<column_grid(b), blk, 0, s>>>(b, static_cast<const float*>(u), static_cast<const float*>(r),
                                                           static_cast<float*>(out), c);
    else
        mg_column_kernel<1><<<column_grid(b), blk, 0, s>>>(b, static_cast<const float*>(r), nullptr, static_cast<float*>(out), c);
    NGB_LAUNCH_CHECK("mg_column_kernel");
    return NGB_OK;
}

int ngb_mg_residual(const ngb_poisson_desc* d, const void* u, const void* r, void* out, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(r && out && r != out && u != out, "r/out must be distinct non-NULL device pointers, u must differ from out");
    const Box    b = box_of(d);
    cudaStream_t s = as_stream(stream);
    const dim3 blk(kZX, kZY);
    if (u)
        mg_column_kernel<2><<<column_grid(b), blk, 0, s>>>(b, static_cast<const float*>(u), static_cast<const float*>(r),
                                                           static_cast<float*>(out), 0.f);
    else
        mg_column_kernel<3><<<column_grid(b), blk, 0, s>>>(b, static_cast<const float*>(r), nullptr, static_cast<float*>(out), 0.f);
    NGB_LAUNCH_CHECK("mg_column_kernel");
    return NGB_OK;
}

int ngb_mg_apply(const ngb_poisson_desc* d, const void* u, void* out, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(u && out && u != out, "u/out must be distinct non-NULL device pointers");
    const Box b = box_of(d);
    mg_column_kernel<4><<<column_grid(b), dim3(kZX, kZY), 0, as_stream(stream)>>>(b, static_cast<const float*>(u), nullptr,
                                                                                    static_cast<float*>(out), 0.f);
    NGB_LAUNCH_CHECK("mg_column_kernel");
    return NGB_OK;
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
