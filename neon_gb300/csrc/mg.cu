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
// One thread per node, x fastest (coalesced rows, the six neighbours of a
// node come from the rows the warp and its neighbours read: L1/L2 hits).
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

// (6 u_c - sum of the six neighbours) / h^2 at an interior node (every neighbour exists)
__device__ __forceinline__ float apply_a(const Box& b, const float* __restrict__ u, int64_t i)
{
    const int64_t sy = b.nx, sz = int64_t(b.nx) * b.ny;
    const float   s = ((__ldg(u + i - 1) + __ldg(u + i + 1)) + (__ldg(u + i - sy) + __ldg(u + i + sy))) +
                    (__ldg(u + i - sz) + __ldg(u + i + sz));
    return __fmul_rn(__fmaf_rn(6.f, __ldg(u + i), -s), b.inv_h2);
}

// mode 0: out = u + c (r - A u); mode 1: out = 2 c r - c^2 A r (two sweeps from zero);
// mode 2: out = r - A u (residual); mode 3: residual with u = 0 (copy of r on Free nodes)
template <int MODE>
__global__ void __launch_bounds__(kMgBX) mg_point_kernel(Box b, const float* __restrict__ u, const float* __restrict__ r,
                                                        float* __restrict__ out, float c)
{
    const int x = blockIdx.x * kMgBX + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= b.nx) return;
    const int64_t i = x + int64_t(b.nx) * (y + int64_t(b.ny) * z);
    if (!interior(b, x, y, z)) {
        out[i] = 0.f;
        return;
    }
    const float ri = __ldg(r + i);
    if (MODE == 0) out[i] = __fmaf_rn(c, ri - apply_a(b, u, i), __ldg(u + i));
    if (MODE == 1) out[i] = __fmaf_rn(-c * c, apply_a(b, r, i), 2.f * c * ri);
    if (MODE == 2) out[i] = ri - apply_a(b, u, i);
    if (MODE == 3) out[i] = ri;
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

__global__ void __launch_bounds__(kMgBX) mg_prolong_add_kernel(Box f, Box c, const float* __restrict__ ec, float* __restrict__ u)
{
    const int x = blockIdx.x * kMgBX + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= f.nx) return;
    const int64_t i = x + int64_t(f.nx) * (y + int64_t(f.ny) * z);
    if (!interior(f, x, y, z)) return;
    const int64_t sy = c.nx, sz = int64_t(c.nx) * c.ny;
    // per axis: one coarse node (even) or the mean of two (odd); fine interior nodes map inside the coarse grid
    const int   x0 = x >> 1, y0 = y >> 1, z0 = z >> 1;
    const int   x1 = x0 + (x & 1), y1 = y0 + (y & 1), z1 = z0 + (z & 1);
    const float wx = (x & 1) ? 0.5f : 1.f, wy = (y & 1) ? 0.5f : 1.f, wz = (z & 1) ? 0.5f : 1.f;
    auto        at = [&](int X, int Y, int Z) { return __ldg(ec + X + sy * Y + sz * Z); };
    float       v = at(x0, y0, z0);
    if (x & 1) v += at(x1, y0, z0);
    float vy = v;
    if (y & 1) {
        float t = at(x0, y1, z0);
        if (x & 1) t += at(x1, y1, z0);
        vy += t;
    }
    float vz = vy;
    if (z & 1) {
        float t = at(x0, y0, z1);
        if (x & 1) t += at(x1, y0, z1);
        if (y & 1) {
            float t2 = at(x0, y1, z1);
            if (x & 1) t2 += at(x1, y1, z1);
            t += t2;
        }
        vz += t;
    }
    u[i] += wx * wy * wz * vz;
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
    if (u)
        mg_point_kernel<0><<<grid_of(b), kMgBX, 0, s>>>(b, static_cast<const float*>(u), static_cast<const float*>(r),
                                                        static_cast<float*>(out), c);
    else
        mg_point_kernel<1><<<grid_of(b), kMgBX, 0, s>>>(b, nullptr, static_cast<const float*>(r), static_cast<float*>(out), c);
    NGB_LAUNCH_CHECK("mg_point_kernel");
    return NGB_OK;
}

int ngb_mg_residual(const ngb_poisson_desc* d, const void* u, const void* r, void* out, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(r && out && r != out && u != out, "r/out must be distinct non-NULL device pointers, u must differ from out");
    const Box    b = box_of(d);
    cudaStream_t s = as_stream(stream);
    if (u)
        mg_point_kernel<2><<<grid_of(b), kMgBX, 0, s>>>(b, static_cast<const float*>(u), static_cast<const float*>(r),
                                                        static_cast<float*>(out), 0.f);
    else
        mg_point_kernel<3><<<grid_of(b), kMgBX, 0, s>>>(b, nullptr, static_cast<const float*>(r), static_cast<float*>(out), 0.f);
    NGB_LAUNCH_CHECK("mg_point_kernel");
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
    const Box f = box_of(fine);
    const Box c{fine->nx / 2, fine->ny / 2, fine->nz / 2, f.inv_h2 * 0.25f};
    mg_prolong_add_kernel<<<grid_of(f), kMgBX, 0, as_stream(stream)>>>(f, c, static_cast<const float*>(ec), static_cast<float*>(u));
    NGB_LAUNCH_CHECK("mg_prolong_add_kernel");
    return NGB_OK;
}

}  // extern "C"
