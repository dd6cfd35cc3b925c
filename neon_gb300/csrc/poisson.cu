// Poisson path: 7-point Laplacian, FP64-accumulated deterministic reductions
// and a mixed-precision (Jacobi-)PCG whose scalars stay on the device.
//
// Compiled with --fmad=false: field updates are the IEEE operation sequence
//   z = T(invdiag * r); p' = z + T(beta) * p; s = (-sum + n p'_c) * (1/h^2)
//   x_lo += T(alpha) p'; r -= T(alpha) s
// that the CPU oracle restates; reductions accumulate in double.
//
// Reductions: every CTA reduces its FP64 partial with warp shuffles and
// shared memory and writes it to a per-CTA slot; the last CTA to take a
// ticket (atomicAdd) sums the slots in CTA order and finalises the scalars.
// No CTA ever waits on another (no spin loops), and the result does not
// depend on which CTA finishes last.
#include "common.cuh"
#include <chrono>
#include <random>
#include <mutex>
#include <vector>

namespace ngb {
namespace {

constexpr int kBX = 256;  // threads per CTA (one row segment)

int sm_count()
{
    static int sms = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    });
    return sms;
}

struct Dom {
    int32_t       nx, ny, nz, xchunks;
    int64_t       segs;  // ny * nz * xchunks
    double        h;
    const int8_t* bd;
    double        invd[7];  // h^2 / n for n valid neighbours (host-computed: no division on the device)
    float         invf[7];  // the same, rounded to float (no FP64 conversion on the device)
    float         ih2_hi, ih2_lo;  // 1/h^2 as a float pair (hi + lo, about 48 bits)
    int32_t       zc;       // planes per CG work item (make_dom: enough items to fill the GPU)
    int32_t       zc_box;   // the same for the 32 x 32 tiles of the box pass A
};

// Dot-product accumulator of one thread. For FP32 operands the exact product
// (Dekker's TwoProduct via fma) is accumulated with Knuth's TwoSum in a float
// pair, about 48 significant bits, without occupying GB300's FP64 pipe; the
// pair becomes a double at the CTA reduction. FP64 operands accumulate in FP64.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<float> {
    float                      s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float a, float b)
    {
        const float p = a * b;
        const float e = __fmaf_rn(a, b, -p);
        const float t = s + p;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (p - bp);
        s = t;
        c = c + (err + e);
    }
    __device__ __forceinline__ double value() const { return double(s) + double(c); }
};
template <>
struct DotAcc<double> {
    double                     s = 0.0;
    __device__ __forceinline__ void   add(double a, double b) { s += a * b; }
    __device__ __forceinline__ double value() const { return s; }
};

Dom make_dom(const ngb_poisson_desc* d)
{
    Dom g{};
    g.nx = d->nx, g.ny = d->ny, g.nz = d->nz;
    g.xchunks = (d->nx + kBX - 1) / kBX;
    g.segs = int64_t(d->ny) * d->nz * g.xchunks;
    g.h = d->h;
    g.bd = d->bd;
    g.invd[0] = 1.0;
    for (int n = 1; n <= 6; n++) g.invd[n] = d->h * d->h / double(n);
    for (int n = 0; n <= 6; n++) g.invf[n] = float(g.invd[n]);
    const double ih2 = 1.0 / (d->h * d->h);
    g.ih2_hi = float(ih2);
    g.ih2_lo = float(ih2 - double(g.ih2_hi));
    // CG work items are 32 x 16 (pass A) column tiles times zc planes: at
    // least four per SM, with chunks as long as that allows (each costs two
    // extra planes of loads at its start)
    const int64_t cols = int64_t((d->nx + 31) / 32) * ((d->ny + 15) / 16);
    g.zc = 64;
    while (g.zc > 8 && cols * ((d->nz + g.zc - 1) / g.zc) < int64_t(sm_count()) * 4) g.zc /= 2;
    const int64_t cols_box = int64_t((d->nx + 31) / 32) * ((d->ny + 31) / 32);
    g.zc_box = 64;
    while (g.zc_box > 8 && cols_box * ((d->nz + g.zc_box - 1) / g.zc_box) < int64_t(sm_count()) * 4) g.zc_box /= 2;
    return g;
}

int grid_for(int64_t segs) { return int(std::min<int64_t>(segs, int64_t(sm_count()) * 8)); }

struct Cell {
    int     x, y, z;
    int64_t i;
};

// Segment -> cell of this thread (x = -1 when past the row end).
__device__ __forceinline__ Cell seg_cell(const Dom& d, int64_t seg)
{
    // 32-bit index arithmetic (segments < 2^31, checked on the host): 64-bit
    // division is a long emulated sequence on the GPU.
    const uint32_t s32 = uint32_t(seg);
    const uint32_t row = s32 / uint32_t(d.xchunks);
    const int      xc = int(s32 - row * uint32_t(d.xchunks));
    Cell           c;
    c.x = xc * kBX + threadIdx.x;
    c.y = int(row % uint32_t(d.ny));
    c.z = int(row / uint32_t(d.ny));
    c.i = c.x + int64_t(d.nx) * (c.y + int64_t(d.ny) * c.z);
    if (c.x >= d.nx) c.x = -1;
    return c;
}

__device__ __forceinline__ bool is_fixed(const Dom& d, int x, int y, int z, int64_t i)
{
    if (d.bd) return d.bd[i] == 0;
    return x == 0 || y == 0 || z == 0 || x == d.nx - 1 || y == d.ny - 1 || z == d.nz - 1;
}

__device__ __forceinline__ int n_valid(const Dom& d, int x, int y, int z)
{
    return (x + 1 < d.nx) + (x > 0) + (y + 1 < d.ny) + (y > 0) + (z + 1 < d.nz) + (z > 0);
}

template <typename T>
__device__ __forceinline__ T invdiag_of(const Dom& d, int x, int y, int z, int64_t i, int jacobi)
{
    if (!jacobi) return T(1);
    if (!d.bd) {  // analytic box: faces are Fixed, every Free cell has six valid neighbours
        if (x == 0 || y == 0 || z == 0 || x == d.nx - 1 || y == d.ny - 1 || z == d.nz - 1) return T(1);
        if constexpr (std::is_same<T, float>::value)
            return d.invf[6];
        else
            return d.invd[6];
    }
    if (is_fixed(d, x, y, z, i)) return T(1);
    // constant indices only: a runtime index into the parameter array would
    // copy it to local memory
    const int n = n_valid(d, x, y, z);
    if constexpr (std::is_same<T, float>::value)
        return n == 6 ? d.invf[6] : n == 5 ? d.invf[5] : n == 4 ? d.invf[4] : n == 3 ? d.invf[3] : n == 2 ? d.invf[2] : n == 1 ? d.invf[1] : d.invf[0];
    else
        return n == 6 ? d.invd[6] : n == 5 ? d.invd[5] : n == 4 ? d.invd[4] : n == 3 ? d.invd[3] : n == 2 ? d.invd[2] : n == 1 ? d.invd[1] : d.invd[0];
}

// Neighbour visitor in the oracle's order +x, -x, +y, -y, +z, -z.
template <typename F>
__device__ __forceinline__ void for_each_ngh(const Dom& d, int x, int y, int z, int64_t i, F f)
{
    const int64_t sy = d.nx, sz = int64_t(d.nx) * d.ny;
    if (x + 1 < d.nx) f(x + 1, y, z, i + 1);
    if (x > 0) f(x - 1, y, z, i - 1);
    if (y + 1 < d.ny) f(x, y + 1, z, i + sy);
    if (y > 0) f(x, y - 1, z, i - sy);
    if (z + 1 < d.nz) f(x, y, z + 1, i + sz);
    if (z > 0) f(x, y, z - 1, i - sz);
}

// ---------------------------------------------------------------- reductions
template <int NS>
__device__ __forceinline__ void cta_sum(double (&v)[NS], double (*sh)[kBX / 32])
{
#pragma unroll
    for (int k = 0; k < NS; k++) {
        double a = v[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = a;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < NS; k++) {
            double a = threadIdx.x < kBX / 32 ? sh[k][threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            v[k] = a;  // valid in thread 0
        }
    }
}

// Writes this CTA's NS sums; returns true in the last CTA, whose thread 0
// then holds in `out` the sums over all CTAs in CTA order.
template <int NS>
__device__ __forceinline__ bool grid_sum(double (&v)[NS], double* partials, unsigned int* ticket, double (&out)[NS])
{
    __shared__ double       sh[NS][kBX / 32];
    __shared__ unsigned int t;
    __shared__ double       fin[NS][kBX];
    cta_sum<NS>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NS; k++) partials[size_t(blockIdx.x) * NS + k] = v[k];
        __threadfence();
        t = atomicAdd(ticket, 1u);
    }
    __syncthreads();
    if (t != gridDim.x - 1) return false;
    __threadfence();
    double acc[NS];
#pragma unroll
    for (int k = 0; k < NS; k++) acc[k] = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kBX)
#pragma unroll
        for (int k = 0; k < NS; k++) acc[k] += __ldcg(partials + size_t(b) * NS + k);
#pragma unroll
    for (int k = 0; k < NS; k++) fin[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = kBX / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
#pragma unroll
            for (int k = 0; k < NS; k++) fin[k][threadIdx.x] += fin[k][threadIdx.x + w];
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < NS; k++) out[k] = fin[k][0];
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// ---------------------------------------------------------------- state
struct CgState {
    double       rz, rz_prev, pAp, alpha, rr, bnorm, rel, tol;
    int32_t      iter, converged, refresh, refresh_every, max_iter, refreshes, last, jacobi;
    unsigned int ticket;
    unsigned int pad;
};

// ---------------------------------------------------------------- kernels
template <typename T>
__global__ void __launch_bounds__(kBX) laplacian_kernel(Dom d, const T* __restrict__ u, T* __restrict__ out)
{
    const T invh2 = T(1.0) / (T(d.h) * T(d.h));
    for (int64_t seg = blockIdx.x; seg < d.segs; seg += gridDim.x) {
        const Cell c = seg_cell(d, seg);
        if (c.x < 0) continue;
        const T uc = u[c.i];
        if (is_fixed(d, c.x, c.y, c.z, c.i)) {
            out[c.i] = uc;
            continue;
        }
        T   sum = T(0);
        int n = 0;
        for_each_ngh(d, c.x, c.y, c.z, c.i, [&](int, int, int, int64_t j) {
            sum = sum + u[j];
            n++;
        });
        out[c.i] = (-sum + T(n) * uc) * invh2;
    }
}

template <typename T>
__global__ void __launch_bounds__(kBX) dot_kernel(int64_t n, const T* __restrict__ a, const T* __restrict__ b, double* result,
                                                  double* partials, unsigned int* ticket)
{
    DotAcc<T> acc;
    for (int64_t i = int64_t(blockIdx.x) * kBX + threadIdx.x; i < n; i += int64_t(gridDim.x) * kBX) acc.add(a[i], b[i]);
    double v[1] = {acc.value()};
    double out[1];
    if (grid_sum<1>(v, partials, ticket, out) && threadIdx.x == 0) *result = out[0];
}

// FCG(1) direction with device scalars (no host round trip): coef = zq /
// pq_prev (0 when zq is NULL: the first direction); p = z - coef p_prev and
// q = az - coef q_prev overwrite z and az; out = {<p, q>, <p, r>}.
__global__ void __launch_bounds__(kBX) fcg_direction_kernel(int64_t n, float* __restrict__ z, float* __restrict__ az,
                                                           const float* __restrict__ pp, const float* __restrict__ qp,
                                                           const float* __restrict__ r, const double* zq, const double* pq_prev,
                                                           double* out, double* partials, unsigned int* ticket)
{
    const bool    first = zq == nullptr;
    const float   coef = first ? 0.f : float(*zq / *pq_prev);
    DotAcc<float> apq, apr;
    const int64_t st = int64_t(gridDim.x) * kBX;
    int64_t       i = int64_t(blockIdx.x) * kBX + threadIdx.x;
    // four elements per trip, all loads first (more bytes in flight per thread)
    for (; i + 3 * st < n; i += 4 * st) {
        float p[4], q[4], rr[4], a[4], b[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            p[k] = z[i + k * st];
            q[k] = az[i + k * st];
            rr[k] = r[i + k * st];
            if (!first) {
                a[k] = pp[i + k * st];
                b[k] = qp[i + k * st];
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (!first) {
                p[k] = __fmaf_rn(-coef, a[k], p[k]);
                q[k] = __fmaf_rn(-coef, b[k], q[k]);
                z[i + k * st] = p[k];
                az[i + k * st] = q[k];
            }
            apq.add(p[k], q[k]);
            apr.add(p[k], rr[k]);
        }
    }
    for (; i < n; i += st) {
        float p = z[i], q = az[i];
        if (!first) {
            p = __fmaf_rn(-coef, pp[i], p);
            q = __fmaf_rn(-coef, qp[i], q);
            z[i] = p;
            az[i] = q;
        }
        apq.add(p, q);
        apr.add(p, r[i]);
    }
    double v[2] = {apq.value(), apr.value()};
    double o[2];
    if (grid_sum<2>(v, partials, ticket, o) && threadIdx.x == 0) {
        out[0] = o[0];
        out[1] = o[1];
    }
}

// FCG(1) update: alpha = pqpr[1] / pqpr[0]; x += alpha p (FP64), r -= alpha q; *rr = <r, r>.
__global__ void __launch_bounds__(kBX) fcg_update_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ p,
                                                        float* __restrict__ r, const float* __restrict__ q,
                                                        const double* pqpr, double* rr, double* partials, unsigned int* ticket)
{
    const double  alpha = pqpr[1] / pqpr[0];
    const float   af = float(alpha);
    DotAcc<float> acc;
    const int64_t st = int64_t(gridDim.x) * kBX;
    int64_t       i = int64_t(blockIdx.x) * kBX + threadIdx.x;
    for (; i + 3 * st < n; i += 4 * st) {
        double xv[4];
        float  pv[4], qv[4], rv[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            xv[k] = x[i + k * st];
            pv[k] = p[i + k * st];
            qv[k] = q[i + k * st];
            rv[k] = r[i + k * st];
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            x[i + k * st] = fma(alpha, double(pv[k]), xv[k]);
            const float ri = __fmaf_rn(-af, qv[k], rv[k]);
            r[i + k * st] = ri;
            acc.add(ri, ri);
        }
    }
    for (; i < n; i += st) {
        x[i] = fma(alpha, double(p[i]), x[i]);
        const float ri = __fmaf_rn(-af, q[i], r[i]);
        r[i] = ri;
        acc.add(ri, ri);
    }
    double v[1] = {acc.value()};
    double o[1];
    if (grid_sum<1>(v, partials, ticket, o) && threadIdx.x == 0) *rr = o[0];
}

// r = T(b - A x_hi) (0 on Fixed rows); sums: |b|^2 over Free rows, r.z, |b - A x|^2.
template <typename T>
__global__ void __launch_bounds__(kBX) cg_init_kernel(Dom d, CgState* st, const T* __restrict__ bvec, const double* __restrict__ xh,
                                                      T* __restrict__ r, T* __restrict__ p, T* __restrict__ xlo,
                                                      double* partials, float* __restrict__ rt_hi, float* __restrict__ rt_lo)
{
    const double invh2 = 1.0 / (d.h * d.h);
    double       v[3] = {0.0, 0.0, 0.0};
    DotAcc<T>    bacc, rzacc;
    for (int64_t seg = blockIdx.x; seg < d.segs; seg += gridDim.x) {
        const Cell c = seg_cell(d, seg);
        if (c.x < 0) continue;
        double rt = 0.0;
        if (!is_fixed(d, c.x, c.y, c.z, c.i)) {
            double sum = 0.0;
            int    n = 0;
            for_each_ngh(d, c.x, c.y, c.z, c.i, [&](int, int, int, int64_t j) {
                sum = sum + xh[j];
                n++;
            });
            const double ax = (-sum + double(n) * xh[c.i]) * invh2;
            rt = double(bvec[c.i]) - ax;
            bacc.add(bvec[c.i], bvec[c.i]);
        }
        const T rc = T(rt);
        r[c.i] = rc;
        p[c.i] = T(0);
        xlo[c.i] = T(0);
        if (rt_hi) {  // FP32 fields: the true residual kept as a float pair for the refreshes
            const float hi = float(rt);
            rt_hi[c.i] = hi;
            rt_lo[c.i] = float(rt - double(hi));
        }
        rzacc.add(rc, T(invdiag_of<T>(d, c.x, c.y, c.z, c.i, st->jacobi) * rc));
        v[2] += rt * rt;
    }
    v[0] = bacc.value();
    v[1] = rzacc.value();
    double out[3];
    if (grid_sum<3>(v, partials, &st->ticket, out) && threadIdx.x == 0) {
        st->bnorm = sqrt(out[0]);
        st->rz = out[1];
        st->rz_prev = 0.0;
        st->rel = st->bnorm > 0 ? sqrt(out[2]) / st->bnorm : 0.0;
        st->iter = 0;
        st->refreshes = 0;
        st->refresh = 0;
        st->last = 0;
        st->converged = (st->bnorm == 0.0 || st->rel <= st->tol) ? 1 : 0;
    }
}

// pass A: beta from device scalars; p' = z + beta p; s = A p'; pAp = <p', s>;
// alpha = rz / pAp. 2.5-D blocking: a CTA takes a 32 x 16 (x, y) tile and
// marches along z through a chunk of d.zc planes; each thread owns the cells
// (x, y) and (x, y + 8) of the tile. Each thread computes p' of its own cells
// once per plane (two loads each); 100 threads also compute the in-plane halo
// into shared memory; the z neighbours stay in registers. So every p' value
// is formed from r and p once per tile instead of once per stencil use.
constexpr int kTX = 32, kTYA = 16, kRY = kTYA / (kBX / kTX);
constexpr int kTY = kBX / kTX;                    // pass B tile height (one column per thread)
constexpr int kHalo = 2 * (kTX + 2) + 2 * kTYA;  // halo cells of one plane of a pass-A tile
static_assert(kRY == 2 && kHalo <= kBX, "tile shape");

__host__ __device__ inline int pass_a_items(const Dom& d)
{
    return ((d.nx + kTX - 1) / kTX) * ((d.ny + kTYA - 1) / kTYA) * ((d.nz + d.zc - 1) / d.zc);
}
__host__ __device__ inline int pass_b_items(const Dom& d)
{
    return ((d.nx + kTX - 1) / kTX) * ((d.ny + kTY - 1) / kTY) * ((d.nz + d.zc - 1) / d.zc);
}

template <typename T>
__device__ __forceinline__ T invdiag6(const Dom& d, int jac)
{
    if (!jac) return T(1);
    if constexpr (std::is_same<T, float>::value)
        return d.invf[6];
    else
        return d.invd[6];
}

// BOX: the analytic box (no boundary array): faces are Fixed, Free cells have
// six valid neighbours, so the Jacobi diagonal of a column depends only on
// whether it lies on an x/y face and on z. Otherwise every value goes through
// invdiag_of / is_fixed (boundary array, Free cells on faces).
template <typename T, bool BOX>
__global__ void __launch_bounds__(kBX) cg_pass_a_kernel(Dom d, CgState* st, const T* __restrict__ r, const T* __restrict__ p_old,
                                                        T* __restrict__ p_new, T* __restrict__ s, double* partials)
{
    if (st->converged) return;
    const int    jac = st->jacobi;
    const double beta = st->rz_prev == 0.0 ? 0.0 : st->rz / st->rz_prev;
    const T      tb = T(beta);
    const T      invh2 = T(1.0) / (T(d.h) * T(d.h));
    const T      dg6 = invdiag6<T>(d, jac);
    __shared__ T planes[2][kTYA + 2][kTX + 2];  // double-buffered: one barrier per plane
    const int    lx = threadIdx.x % kTX, ly0 = threadIdx.x / kTX;  // rows ly0 and ly0 + 8 of the tile
    // this thread's halo cell (threads < kHalo), in tile coordinates
    int        hx = 0, hy = 0;
    const bool halo = threadIdx.x < kHalo;
    if (threadIdx.x < kTX + 2) {
        hx = threadIdx.x - 1, hy = -1;
    } else if (threadIdx.x < 2 * (kTX + 2)) {
        hx = threadIdx.x - (kTX + 2) - 1, hy = kTYA;
    } else if (halo) {
        const int k = threadIdx.x - 2 * (kTX + 2);
        hx = (k & 1) ? kTX : -1, hy = k >> 1;
    }
    const int     ntx = (d.nx + kTX - 1) / kTX, nty = (d.ny + kTYA - 1) / kTYA;
    const int     items = pass_a_items(d);
    const int64_t pl = int64_t(d.nx) * d.ny;
    DotAcc<T>     acc;
    // p' of a column at plane zz from its raw values; 0 outside the grid
    auto pn = [&](bool ok, bool face, int64_t col, int xx, int yy, int zz, T rv, T pv) -> T {
        if (!ok || zz < 0 || zz >= d.nz) return T(0);
        T dgv;
        if constexpr (BOX)
            dgv = (face || zz == 0 || zz == d.nz - 1) ? T(1) : dg6;
        else
            dgv = invdiag_of<T>(d, xx, yy, zz, col + zz * pl, jac);
        return T(dgv * rv) + tb * pv;
    };
    // raw (r, p) of a column at plane zz; zeros outside the grid
    auto load = [&](bool ok, int64_t col, int zz, T& rv, T& pv) {
        if (ok && zz >= 0 && zz < d.nz) {
            rv = r[col + zz * pl];
            pv = p_old[col + zz * pl];
        } else {
            rv = T(0), pv = T(0);
        }
    };
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int tx = item % ntx, rest = item / ntx, ty = rest % nty, zc = rest / nty;
        const int x = tx * kTX + lx, z0 = zc * d.zc, z1 = min(z0 + d.zc, d.nz);
        const int gx = tx * kTX + hx, gy = ty * kTYA + hy;
        const bool    hown = halo && gx >= 0 && gy >= 0 && gx < d.nx && gy < d.ny;
        const int64_t hc = hown ? gx + int64_t(d.nx) * gy : 0;
        const bool    hface = gx == 0 || gy == 0 || gx == d.nx - 1 || gy == d.ny - 1;
        int     y[kRY];
        bool    own[kRY], oface[kRY];
        int64_t oc[kRY];
        T       pprev[kRY], pc[kRY], r1[kRY], p1[kRY];
#pragma unroll
        for (int c = 0; c < kRY; c++) {
            y[c] = ty * kTYA + ly0 + 8 * c;
            own[c] = x < d.nx && y[c] < d.ny;
            oc[c] = own[c] ? x + int64_t(d.nx) * y[c] : 0;
            oface[c] = x == 0 || y[c] == 0 || x == d.nx - 1 || y[c] == d.ny - 1;
            T ra, pa, rb, pb;
            load(own[c], oc[c], z0 - 1, ra, pa);
            load(own[c], oc[c], z0, rb, pb);
            load(own[c], oc[c], z0 + 1, r1[c], p1[c]);
            pprev[c] = pn(own[c], oface[c], oc[c], x, y[c], z0 - 1, ra, pa);
            pc[c] = pn(own[c], oface[c], oc[c], x, y[c], z0, rb, pb);
        }
        T hr, hp;
        load(hown, hc, z0, hr, hp);
        // the previous item's last plane may share a buffer with this item's first
        __syncthreads();
        for (int z = z0; z < z1; z++) {
            // one plane of lookahead: these loads are used in the next iteration
            T r2[kRY], p2[kRY], hr2, hp2, pnext[kRY];
#pragma unroll
            for (int c = 0; c < kRY; c++) {
                load(own[c], oc[c], z + 2, r2[c], p2[c]);
                pnext[c] = pn(own[c], oface[c], oc[c], x, y[c], z + 1, r1[c], p1[c]);
            }
            load(hown, hc, z + 1, hr2, hp2);
            const T hv = pn(hown, hface, hc, gx, gy, z, hr, hp);
            // buffer z & 1 was last read in iteration z - 2, before the barrier of iteration z - 1
            T (*plane)[kTX + 2] = planes[z & 1];
#pragma unroll
            for (int c = 0; c < kRY; c++) plane[ly0 + 8 * c + 1][lx + 1] = pc[c];
            if (halo) plane[hy + 1][hx + 1] = hv;
            __syncthreads();
#pragma unroll
            for (int c = 0; c < kRY; c++) {
                if (!own[c]) continue;
                const int     ly = ly0 + 8 * c;
                const int64_t i = oc[c] + int64_t(z) * pl;
                T             sc;
                const bool    inner = !oface[c] && z >= 1 && z < d.nz - 1;
                if (BOX || (!d.bd && inner)) {
                    if (inner) {
                        T sum = T(0);
                        sum = sum + plane[ly + 1][lx + 2];
                        sum = sum + plane[ly + 1][lx];
                        sum = sum + plane[ly + 2][lx + 1];
                        sum = sum + plane[ly][lx + 1];
                        sum = sum + pnext[c];
                        sum = sum + pprev[c];
                        sc = (-sum + T(6) * pc[c]) * invh2;
                    } else {
                        sc = pc[c];  // Fixed face row
                    }
                } else if (is_fixed(d, x, y[c], z, i)) {
                    sc = pc[c];
                } else {  // neighbours in the oracle's order +x, -x, +y, -y, +z, -z, valid ones only
                    T   sum = T(0);
                    int n = 0;
                    if (x + 1 < d.nx) sum = sum + plane[ly + 1][lx + 2], n++;
                    if (x > 0) sum = sum + plane[ly + 1][lx], n++;
                    if (y[c] + 1 < d.ny) sum = sum + plane[ly + 2][lx + 1], n++;
                    if (y[c] > 0) sum = sum + plane[ly][lx + 1], n++;
                    if (z + 1 < d.nz) sum = sum + pnext[c], n++;
                    if (z > 0) sum = sum + pprev[c], n++;
                    sc = (-sum + T(n) * pc[c]) * invh2;
                }
                p_new[i] = pc[c];
                s[i] = sc;
                acc.add(pc[c], sc);
            }
#pragma unroll
            for (int c = 0; c < kRY; c++) {
                pprev[c] = pc[c];
                pc[c] = pnext[c];
                r1[c] = r2[c], p1[c] = p2[c];
            }
            hr = hr2, hp = hp2;
        }
    }
    double v[1] = {acc.value()};
    double out[1];
    if (grid_sum<1>(v, partials, &st->ticket, out) && threadIdx.x == 0) {
        st->pAp = out[0];
        st->alpha = st->rz / out[0];
    }
}

// pass A for the analytic box with float fields and fewer than 2^31 cells:
// the planes and arithmetic of cg_pass_a_kernel<float, true> (so the outputs
// are the same bits) on taller tiles, 32 x 32 columns per CTA with four cells
// per thread (rows ly0 + 8c), so one barrier per plane serves four cells and
// the halo is 13 % of a tile instead of 20 %; 32-bit cell indices stepped one
// plane at a time, one uniform validity test per plane, columns outside the
// grid parked on cell 0 (read, never used or written); 64 registers, four
// CTAs per SM.
constexpr int kBoxR = 4, kBoxTY = 8 * kBoxR, kBoxHalo = 2 * (kTX + 2) + 2 * kBoxTY;
static_assert(kBoxHalo <= kBX, "box halo");

__host__ __device__ inline int pass_a_box_items(const Dom& d)
{
    return ((d.nx + kTX - 1) / kTX) * ((d.ny + kBoxTY - 1) / kBoxTY) * ((d.nz + d.zc_box - 1) / d.zc_box);
}

__global__ void __launch_bounds__(kBX, 4) cg_pass_a_box_kernel(Dom d, CgState* st, const float* __restrict__ r,
                                                               const float* __restrict__ p_old, float* __restrict__ p_new,
                                                               float* __restrict__ s, double* partials)
{
    constexpr int R = kBoxR, TY = kBoxTY;
    if (st->converged) return;
    const int    jac = st->jacobi;
    const double beta = st->rz_prev == 0.0 ? 0.0 : st->rz / st->rz_prev;
    const float  tb = float(beta);
    const float  invh2 = 1.0f / (float(d.h) * float(d.h));
    const float  dg6 = invdiag6<float>(d, jac);
    __shared__ float planes[2][TY + 2][kTX + 2];
    const int    lx = threadIdx.x % kTX, ly0 = threadIdx.x / kTX;
    int        hx = 0, hy = 0;
    const bool halo = threadIdx.x < kBoxHalo;
    if (threadIdx.x < kTX + 2) {
        hx = threadIdx.x - 1, hy = -1;
    } else if (threadIdx.x < 2 * (kTX + 2)) {
        hx = threadIdx.x - (kTX + 2) - 1, hy = TY;
    } else if (halo) {
        const int k = threadIdx.x - 2 * (kTX + 2);
        hx = (k & 1) ? kTX : -1, hy = k >> 1;
    }
    const int     ntx = (d.nx + kTX - 1) / kTX, nty = (d.ny + TY - 1) / TY;
    const int     items = pass_a_box_items(d);
    const int     pl = d.nx * d.ny;
    DotAcc<float> acc;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int tx = item % ntx, rest = item / ntx, ty = rest % nty, zi = rest / nty;
        const int x = tx * kTX + lx, z0 = zi * d.zc_box, z1 = min(z0 + d.zc_box, d.nz);
        bool      own[R], fc[R];
        int       stc[R], ix[R];
        float     dg[R];
#pragma unroll
        for (int c = 0; c < R; c++) {
            const int y = ty * TY + ly0 + 8 * c;
            own[c] = x < d.nx && y < d.ny;
            fc[c] = x == 0 || x == d.nx - 1 || y == 0 || y == d.ny - 1;
            stc[c] = own[c] ? pl : 0;
            ix[c] = (own[c] ? x + d.nx * y : 0) + z0 * stc[c];
            dg[c] = fc[c] ? 1.f : dg6;
        }
        const int   gx = tx * kTX + hx, gy = ty * TY + hy;
        const bool  hown = halo && gx >= 0 && gy >= 0 && gx < d.nx && gy < d.ny;
        const bool  hface = gx == 0 || gy == 0 || gx == d.nx - 1 || gy == d.ny - 1;
        const int   sth = hown ? pl : 0;
        int         ih = (hown ? gx + d.nx * gy : 0) + z0 * sth;
        const float dgh = hface ? 1.f : dg6;
        // p' = dgv r + tb p (dgv = 1 on the faces), 0 outside the grid
        float pprev[R], pc[R], r1[R], p1[R];
#pragma unroll
        for (int c = 0; c < R; c++) {
            pprev[c] = 0.f, r1[c] = 0.f, p1[c] = 0.f;
            if (z0 >= 1) {
                const float v = float(((z0 - 1 == 0) ? 1.f : dg[c]) * r[ix[c] - stc[c]]) + tb * p_old[ix[c] - stc[c]];
                pprev[c] = own[c] ? v : 0.f;
            }
            const float v = float(((z0 == 0 || z0 == d.nz - 1) ? 1.f : dg[c]) * r[ix[c]]) + tb * p_old[ix[c]];
            pc[c] = own[c] ? v : 0.f;
            if (z0 + 1 < d.nz) r1[c] = r[ix[c] + stc[c]], p1[c] = p_old[ix[c] + stc[c]];
        }
        float hr = r[ih], hp = p_old[ih];
        // the previous item's last plane may share a buffer with this item's first
        __syncthreads();
        for (int z = z0; z < z1; z++) {
            // one plane of lookahead: these loads are used in the next iteration
            float r2[R], p2[R], hr2 = 0.f, hp2 = 0.f;
#pragma unroll
            for (int c = 0; c < R; c++) {
                r2[c] = 0.f, p2[c] = 0.f;
                if (z + 2 < d.nz) r2[c] = r[ix[c] + 2 * stc[c]], p2[c] = p_old[ix[c] + 2 * stc[c]];
            }
            if (z + 1 < d.nz) hr2 = r[ih + sth], hp2 = p_old[ih + sth];
            const bool zn = z + 1 == d.nz - 1, zin = z + 1 < d.nz;
            float      pnext[R];
#pragma unroll
            for (int c = 0; c < R; c++) {
                const float v = float((zn ? 1.f : dg[c]) * r1[c]) + tb * p1[c];
                pnext[c] = (own[c] && zin) ? v : 0.f;
            }
            const bool  zf = z == 0 || z == d.nz - 1;
            const float hvv = float((zf ? 1.f : dgh) * hr) + tb * hp;
            // buffer z & 1 was last read in iteration z - 2, before the barrier of iteration z - 1
            float (*plane)[kTX + 2] = planes[z & 1];
#pragma unroll
            for (int c = 0; c < R; c++) plane[ly0 + 8 * c + 1][lx + 1] = pc[c];
            if (halo) plane[hy + 1][hx + 1] = hown ? hvv : 0.f;
            __syncthreads();
#pragma unroll
            for (int c = 0; c < R; c++) {
                const int ly = ly0 + 8 * c;
                // neighbours in the oracle's order +x, -x, +y, -y, +z, -z
                float sum = 0.f;
                sum = sum + plane[ly + 1][lx + 2];
                sum = sum + plane[ly + 1][lx];
                sum = sum + plane[ly + 2][lx + 1];
                sum = sum + plane[ly][lx + 1];
                sum = sum + pnext[c];
                sum = sum + pprev[c];
                const float sc = (fc[c] || zf) ? pc[c] : (-sum + 6.f * pc[c]) * invh2;  // Fixed face rows: s = p'
                if (own[c]) {
                    p_new[ix[c]] = pc[c], s[ix[c]] = sc;
                    acc.add(pc[c], sc);
                }
                ix[c] += stc[c];
                pprev[c] = pc[c], pc[c] = pnext[c], r1[c] = r2[c], p1[c] = p2[c];
            }
            ih += sth;
            hr = hr2, hp = hp2;
        }
    }
    double v[1] = {acc.value()};
    double out[1];
    if (grid_sum<1>(v, partials, &st->ticket, out) && threadIdx.x == 0) {
        st->pAp = out[0];
        st->alpha = st->rz / out[0];
    }
}

// pass B: x_lo += alpha p; r -= alpha s; rz' = <r, z>; rr = <r, r>. Work
// items of 32 x 8 columns and chunks of d.zc planes: each thread
// walks its column with a running index, the loads of the next plane in
// flight while the current one is updated; BOX as in pass A.
template <typename T, bool BOX>
__global__ void __launch_bounds__(kBX) cg_pass_b_kernel(Dom d, CgState* st, T* __restrict__ xlo, const T* __restrict__ p,
                                                        T* __restrict__ r, const T* __restrict__ s, double* partials,
                                                        cudaGraphConditionalHandle refresh_if, int use_if)
{
    if (st->converged) return;
    const int     jac = st->jacobi;
    const T       ta = T(st->alpha);
    const T       dg6 = invdiag6<T>(d, jac);
    const int     lx = threadIdx.x % kTX, ly = threadIdx.x / kTX;
    const int     ntx = (d.nx + kTX - 1) / kTX, nty = (d.ny + kTY - 1) / kTY;
    const int     items = pass_b_items(d);
    const int64_t pl = int64_t(d.nx) * d.ny;
    DotAcc<T>     a0, a1;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int tx = item % ntx, rest = item / ntx, ty = rest % nty, zc = rest / nty;
        const int x = tx * kTX + lx, y = ty * kTY + ly, z0 = zc * d.zc, z1 = min(z0 + d.zc, d.nz);
        if (x >= d.nx || y >= d.ny) continue;  // no barrier in this kernel
        const bool oface = x == 0 || y == 0 || x == d.nx - 1 || y == d.ny - 1;
        int64_t    i = x + int64_t(d.nx) * y + int64_t(z0) * pl;
        T          xv = xlo[i], pv = p[i], rv = r[i], sv = s[i];
        for (int z = z0; z < z1; z++, i += pl) {
            T xn = T(0), pn = T(0), rn = T(0), sn = T(0);
            if (z + 1 < z1) xn = xlo[i + pl], pn = p[i + pl], rn = r[i + pl], sn = s[i + pl];
            xlo[i] = xv + ta * pv;
            const T rnew = rv - ta * sv;
            r[i] = rnew;
            T dgv;
            if constexpr (BOX)
                dgv = (oface || z == 0 || z == d.nz - 1) ? T(1) : dg6;
            else
                dgv = invdiag_of<T>(d, x, y, z, i, jac);
            const T zz = T(dgv * rnew);
            a0.add(rnew, zz);
            a1.add(rnew, rnew);
            xv = xn, pv = pn, rv = rn, sv = sn;
        }
    }
    double v[2] = {a0.value(), a1.value()};
    double out[2];
    if (grid_sum<2>(v, partials, &st->ticket, out) && threadIdx.x == 0) {
        st->rz_prev = st->rz;
        st->rz = out[0];
        st->rr = out[1];
        st->iter += 1;
        const bool want = (st->iter % st->refresh_every == 0) || (sqrt(out[1]) / st->bnorm <= st->tol);
        st->last = st->iter >= st->max_iter ? 1 : 0;
        st->refresh = (want || st->last) ? 1 : 0;
        // inside the solve graph: the refresh kernels run only when wanted
        if (use_if) cudaGraphSetConditional(refresh_if, unsigned(st->refresh));
    }
}

// refresh, part 1: x_hi += x_lo; x_lo = 0.
template <typename T>
__global__ void __launch_bounds__(kBX) cg_refresh1_kernel(Dom d, const CgState* st, double* __restrict__ xh, T* __restrict__ xlo)
{
    if (st->converged || !st->refresh) return;
    for (int64_t seg = blockIdx.x; seg < d.segs; seg += gridDim.x) {
        const Cell c = seg_cell(d, seg);
        if (c.x < 0) continue;
        xh[c.i] = xh[c.i] + double(xlo[c.i]);
        xlo[c.i] = T(0);
    }
}

// refresh, part 2: r = T(b - A x_hi); rz = <r, z>; true relative residual.
template <typename T>
__global__ void __launch_bounds__(kBX) cg_refresh2_kernel(Dom d, CgState* st, const T* __restrict__ bvec,
                                                          const double* __restrict__ xh, T* __restrict__ r, double* partials)
{
    if (st->converged || !st->refresh) return;
    const double invh2 = 1.0 / (d.h * d.h);
    const int    jac = st->jacobi;
    double       v[2] = {0.0, 0.0};
    DotAcc<T>    rzacc;
    for (int64_t seg = blockIdx.x; seg < d.segs; seg += gridDim.x) {
        const Cell c = seg_cell(d, seg);
        if (c.x < 0) continue;
        double rt = 0.0;
        if (!is_fixed(d, c.x, c.y, c.z, c.i)) {
            double sum = 0.0;
            int    n = 0;
            for_each_ngh(d, c.x, c.y, c.z, c.i, [&](int, int, int, int64_t j) {
                sum = sum + xh[j];
                n++;
            });
            rt = double(bvec[c.i]) - (-sum + double(n) * xh[c.i]) * invh2;
        }
        const T rc = T(rt);
        r[c.i] = rc;
        rzacc.add(rc, T(invdiag_of<T>(d, c.x, c.y, c.z, c.i, jac) * rc));
        v[1] += rt * rt;
    }
    v[0] = rzacc.value();
    double out[2];
    if (grid_sum<2>(v, partials, &st->ticket, out) && threadIdx.x == 0) {
        st->rz = out[0];
        st->rel = sqrt(out[1]) / st->bnorm;
        st->refreshes += 1;
        st->refresh = 0;
        if (st->rel <= st->tol)
            st->converged = 1;
        else if (st->last)
            st->converged = 2;
    }
}

// Float-pair arithmetic (about 48 significant bits on the FP32 pipe): Knuth's
// TwoSum, Dekker's TwoProduct by fma, and the pair sum normalised.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b)
{
    const float s = a + b, bb = s - a;
    return FF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF ff_norm(float hi, float lo)
{
    const float s = hi + lo;
    return FF{s, lo - (s - hi)};
}
__device__ __forceinline__ FF ff_add(FF a, float b)
{
    const FF t = two_sum(a.hi, b);
    return ff_norm(t.hi, t.lo + a.lo);
}

// Refresh for FP32 fields, incremental: the true residual b - A x_hi is kept
// as a float pair (rt_hi, rt_lo) since the start of the solve; folding x_lo
// into x_hi changes it by -A x_lo, computed here in float-pair arithmetic
// (A x_lo is small against b - A x_hi only near convergence, where the pair's
// 48 bits keep it exact to far below the tolerance). So the refresh needs
// two FP64 operations per cell (x_hi += x_lo) instead of an FP64 stencil of
// x_hi, which GB300's FP64 rate made the largest cost of a refresh. Then
// r = rt_hi, rz = <r, z>, rel = |rt| / |b|; x_lo is cleared by the next
// kernel (cells here read their neighbours' x_lo).
__global__ void __launch_bounds__(kBX) cg_refresh_ff_kernel(Dom d, CgState* st, double* __restrict__ xh, const float* __restrict__ xlo,
                                                            float* __restrict__ r, float* __restrict__ rt_hi,
                                                            float* __restrict__ rt_lo, double* partials)
{
    if (st->converged || !st->refresh) return;
    const int     jac = st->jacobi;
    double        v[2] = {0.0, 0.0};
    DotAcc<float> rzacc, rracc;
    for (int64_t seg = blockIdx.x; seg < d.segs; seg += gridDim.x) {
        const Cell c = seg_cell(d, seg);
        if (c.x < 0) continue;
        const float xc = xlo[c.i];
        xh[c.i] = xh[c.i] + double(xc);
        float rh = 0.f;
        if (!is_fixed(d, c.x, c.y, c.z, c.i)) {  // Fixed cells keep r = 0
            // A x_lo = (n x_c - sum of the valid neighbours) / h^2, as a float pair
            int n = 0;
            for_each_ngh(d, c.x, c.y, c.z, c.i, [&](int, int, int, int64_t) { n++; });
            const float p = float(n) * xc;
            FF          a{p, __fmaf_rn(float(n), xc, -p)};
            for_each_ngh(d, c.x, c.y, c.z, c.i, [&](int, int, int, int64_t j) { a = ff_add(a, -xlo[j]); });
            const float ph = a.hi * d.ih2_hi;
            const float pl = __fmaf_rn(a.hi, d.ih2_hi, -ph) + (a.hi * d.ih2_lo + a.lo * d.ih2_hi);
            // rt -= A x_lo
            const FF t = two_sum(rt_hi[c.i], -ph);
            const FF rt = ff_norm(t.hi, t.lo + (rt_lo[c.i] - pl));
            rt_hi[c.i] = rt.hi;
            rt_lo[c.i] = rt.lo;
            rh = rt.hi;
        }
        r[c.i] = rh;
        rzacc.add(rh, float(invdiag_of<float>(d, c.x, c.y, c.z, c.i, jac) * rh));
        rracc.add(rh, rh);
    }
    v[0] = rzacc.value();
    v[1] = rracc.value();
    double out[2];
    if (grid_sum<2>(v, partials, &st->ticket, out) && threadIdx.x == 0) {
        st->rz = out[0];
        st->rel = sqrt(out[1]) / st->bnorm;
        st->refreshes += 1;
        st->refresh = 0;
        if (st->rel <= st->tol)
            st->converged = 1;
        else if (st->last)
            st->converged = 2;
    }
}

// x_lo = 0 after an incremental refresh (a separate launch: the refresh reads
// neighbours' x_lo). Runs whenever the refresh ran: its condition is the IF
// node's, not st->refresh, which the refresh has cleared.
__global__ void __launch_bounds__(kBX) cg_clear_xlo_kernel(int64_t n, float* __restrict__ xlo)
{
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) xlo[i] = 0.f;
}

__global__ void rhs_kernel(Dom d, int field, const double* __restrict__ centres, const double* __restrict__ amps, double sigma,
                           void* f)
{
    const double inv2s2 = 1.0 / (2.0 * sigma * sigma);
    for (int64_t seg = blockIdx.x; seg < d.segs; seg += gridDim.x) {
        const Cell c = seg_cell(d, seg);
        if (c.x < 0) continue;
        double v = 0.0;
        for (int k = 0; k < 8; k++) {
            const double dx = c.x - centres[3 * k], dy = c.y - centres[3 * k + 1], dz = c.z - centres[3 * k + 2];
            v += amps[k] * exp(-(dx * dx + dy * dy + dz * dz) * inv2s2);
        }
        if (field == NGB_STORE_F64)
            static_cast<double*>(f)[c.i] = v;
        else
            static_cast<float*>(f)[c.i] = float(v);
    }
}

// ---------------------------------------------------------------- host helpers
int validate(const ngb_poisson_desc* d)
{
    NGB_CHECK_ARG(d, "desc is NULL");
    NGB_CHECK_ARG(d->nx >= 1 && d->ny >= 1 && d->nz >= 1, "dims must be positive");
    NGB_CHECK_ARG(d->field == NGB_STORE_F32 || d->field == NGB_STORE_F64, "field must be NGB_STORE_F32 or NGB_STORE_F64");
    NGB_CHECK_ARG(d->h > 0, "h must be positive");
    NGB_CHECK_ARG(make_dom(d).segs < (int64_t(1) << 31), "grid too large (ny * nz * ceil(nx / 256) >= 2^31)");
    NGB_CHECK_ARG(int64_t((d->nx + kTX - 1) / kTX) * ((d->ny + kTY - 1) / kTY) * ((d->nz + 7) / 8) < (int64_t(1) << 31),
                  "grid too large for the CG tiling");
    return NGB_OK;
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct Workspace {
    CgState* st;
    double*  partials;
    void *   r, *p0, *p1, *s, *xlo;
    float *  rt_hi, *rt_lo;  // FP32 fields: the true residual as a float pair (null for FP64 fields)
    size_t   bytes;
};

Workspace layout(const ngb_poisson_desc* d, void* base)
{
    const size_t V = size_t(d->nx) * d->ny * d->nz;
    const size_t esz = d->field == NGB_STORE_F64 ? 8 : 4;
    const int    grid = grid_for(make_dom(d).segs);
    Workspace    w{};
    char*        p = static_cast<char*>(base);
    size_t       off = 0;
    w.st = reinterpret_cast<CgState*>(p + off);
    off += align256(sizeof(CgState));
    w.partials = reinterpret_cast<double*>(p + off);
    off += align256(size_t(grid) * 3 * sizeof(double));
    void** fields[5] = {&w.r, &w.p0, &w.p1, &w.s, &w.xlo};
    for (auto f : fields) {
        *f = p + off;
        off += align256(V * esz);
    }
    if (d->field != NGB_STORE_F64) {
        w.rt_hi = reinterpret_cast<float*>(p + off);
        off += align256(V * 4);
        w.rt_lo = reinterpret_cast<float*>(p + off);
        off += align256(V * 4);
    }
    w.bytes = off;
    return w;
}

// pass A launch: the 32-bit-index box kernel where it applies
template <typename T>
void launch_pass_a(const Dom& d, int grid_a, CgState* st, const T* r, const T* pa, T* pb, T* sv, double* partials, cudaStream_t s)
{
    if (d.bd) {
        cg_pass_a_kernel<T, false><<<grid_a, kBX, 0, s>>>(d, st, r, pa, pb, sv, partials);
        return;
    }
    if constexpr (std::is_same<T, float>::value) {
        if (int64_t(d.nx) * d.ny * d.nz < (int64_t(1) << 31)) {
            // four CTAs per SM, no more than the partials hold (grid_a, the other kernels' grid cap)
            const int g = std::min(std::min(grid_a, 4 * sm_count()), pass_a_box_items(d));
            cg_pass_a_box_kernel<<<g, kBX, 0, s>>>(d, st, r, pa, pb, sv, partials);
            return;
        }
    }
    cg_pass_a_kernel<T, true><<<grid_a, kBX, 0, s>>>(d, st, r, pa, pb, sv, partials);
}

template <typename T>
int solve_t(const ngb_poisson_desc* desc, const T* b, double* x, const Workspace& w, const ngb_cg_params* prm,
            ngb_cg_result* res, cudaStream_t s)
{
    const Dom d = make_dom(desc);
    const int grid = grid_for(d.segs);
    CgState   init{};
    init.tol = prm->tol;
    init.refresh_every = prm->refresh_every;
    init.max_iter = prm->max_iter;
    init.jacobi = prm->jacobi ? 1 : 0;
    NGB_CUDA_TRY(cudaMemcpyAsync(w.st, &init, sizeof(CgState), cudaMemcpyHostToDevice, s));
    T *r = static_cast<T*>(w.r), *p0 = static_cast<T*>(w.p0), *p1 = static_cast<T*>(w.p1), *sv = static_cast<T*>(w.s),
      *xlo = static_cast<T*>(w.xlo);
    const auto t0 = std::chrono::steady_clock::now();
    cg_init_kernel<T><<<grid, kBX, 0, s>>>(d, w.st, b, x, r, p0, xlo, w.partials, w.rt_hi, w.rt_lo);
    NGB_LAUNCH_CHECK("cg_init_kernel");
    NGB_CUDA_TRY(cudaMemsetAsync(p1, 0, size_t(desc->nx) * desc->ny * desc->nz * sizeof(T), s));

    // the two passes: no more CTAs than work items (partials hold `grid` entries)
    const int grid_a = std::min(grid, pass_a_items(d)), grid_b = std::min(grid, pass_b_items(d));
    // Capture `check_every` iterations (rounded up to even: p ping-pongs) once.
    // Each iteration is pass A, pass B and an IF node holding the two refresh
    // kernels, whose condition pass B sets: they launch on refresh iterations only.
    const int    per = std::max(2, (prm->check_every + 1) / 2 * 2);
    cudaStream_t cs, cs_body;
    NGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    if (cudaStreamCreateWithFlags(&cs_body, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(cs);
        set_error("cudaStreamCreateWithFlags failed");
        return NGB_ERR_CUDA;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int it = 0; it < per && e == cudaSuccess; it++) {
            T* pa = (it % 2 == 0) ? p0 : p1;
            T* pb = (it % 2 == 0) ? p1 : p0;
            cudaGraphConditionalHandle h{};
            e = cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault);
            if (e != cudaSuccess) break;
            launch_pass_a<T>(d, grid_a, w.st, r, pa, pb, sv, w.partials, cs);
            if (d.bd)
                cg_pass_b_kernel<T, false><<<grid_b, kBX, 0, cs>>>(d, w.st, xlo, pb, r, sv, w.partials, h, 1);
            else
                cg_pass_b_kernel<T, true><<<grid_b, kBX, 0, cs>>>(d, w.st, xlo, pb, r, sv, w.partials, h, 1);
            cudaStreamCaptureStatus cst;
            const cudaGraphNode_t*  deps = nullptr;
            size_t                  ndeps = 0;
            e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, nullptr, &deps, nullptr, &ndeps);
            if (e != cudaSuccess) break;
            cudaGraphNodeParams np{};
            np.type = cudaGraphNodeTypeConditional;
            np.conditional.handle = h;
            np.conditional.type = cudaGraphCondTypeIf;
            np.conditional.size = 1;
            cudaGraphNode_t node;
            e = cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &np);
            if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
            if (e == cudaSuccess)
                e = cudaStreamBeginCaptureToGraph(cs_body, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                if constexpr (std::is_same<T, float>::value) {  // incremental float-pair refresh
                    cg_refresh_ff_kernel<<<grid, kBX, 0, cs_body>>>(d, w.st, x, xlo, r, w.rt_hi, w.rt_lo, w.partials);
                    const int64_t V = int64_t(desc->nx) * desc->ny * desc->nz;
                    cg_clear_xlo_kernel<<<int(std::min<int64_t>((V + kBX - 1) / kBX, int64_t(sm_count()) * 8)), kBX, 0, cs_body>>>(V,
                                                                                                                           xlo);
                } else {
                    cg_refresh1_kernel<T><<<grid, kBX, 0, cs_body>>>(d, w.st, x, xlo);
                    cg_refresh2_kernel<T><<<grid, kBX, 0, cs_body>>>(d, w.st, b, x, r, w.partials);
                }
                cudaGraph_t body = nullptr;
                e = cudaStreamEndCapture(cs_body, &body);
            }
        }
        cudaGraph_t captured = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cs, &captured);
        if (e == cudaSuccess) e = e2;
    }
    cudaStreamDestroy(cs_body);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        set_error("CG graph capture failed: %s", cudaGetErrorString(e));
        return NGB_ERR_CUDA;
    }
    cudaGraphExec_t exec;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error("CG graph instantiate failed: %s", cudaGetErrorString(e));
        return NGB_ERR_CUDA;
    }
    // pinned 4-byte landing slot of the stop-flag polls: one per host thread,
    // allocated on its first solve and kept
    static thread_local int32_t* flag = nullptr;
    if (!flag) {
        e = cudaMallocHost(&flag, sizeof(int32_t));
        if (e != cudaSuccess) {
            flag = nullptr;
            cudaGraphExecDestroy(exec);
            set_error("cudaMallocHost failed: %s", cudaGetErrorString(e));
            return NGB_ERR_CUDA;
        }
    }
    int rc = NGB_OK;
    const int max_launches = (prm->max_iter + per - 1) / per + 1;
    for (int l = 0; l <= max_launches; l++) {
        e = cudaMemcpyAsync(flag, &w.st->converged, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("CG poll failed: %s", cudaGetErrorString(e));
            rc = NGB_ERR_CUDA;
            break;
        }
        if (*flag) break;
        e = cudaGraphLaunch(exec, s);
        if (e != cudaSuccess) {
            set_error("CG graph launch failed: %s", cudaGetErrorString(e));
            rc = NGB_ERR_CUDA;
            break;
        }
    }
    const auto t1 = std::chrono::steady_clock::now();
    cudaGraphExecDestroy(exec);
    if (rc) return rc;
    CgState out;
    NGB_CUDA_TRY(cudaMemcpyAsync(&out, w.st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    NGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (res) {
        res->iterations = out.iter;
        res->converged = out.converged == 1;
        res->refreshes = out.refreshes;
        res->rel_residual = out.rel;
        res->seconds = std::chrono::duration<double>(t1 - t0).count();
    }
    return NGB_OK;
}

template <typename T>
int time_passes_t(const ngb_poisson_desc* desc, const T* b, double* x, const Workspace& w, int reps, float* ms, cudaStream_t s)
{
    const Dom d = make_dom(desc);
    const int grid = grid_for(d.segs);
    CgState   init{};
    init.tol = 0.0;                  // never converged while timing
    init.refresh_every = 1 << 30;    // no refresh inside the timed passes
    init.max_iter = 1 << 30;
    init.jacobi = 1;
    NGB_CUDA_TRY(cudaMemcpyAsync(w.st, &init, sizeof(CgState), cudaMemcpyHostToDevice, s));
    T *r = static_cast<T*>(w.r), *p0 = static_cast<T*>(w.p0), *p1 = static_cast<T*>(w.p1), *sv = static_cast<T*>(w.s),
      *xlo = static_cast<T*>(w.xlo);
    cg_init_kernel<T><<<grid, kBX, 0, s>>>(d, w.st, b, x, r, p0, xlo, w.partials, w.rt_hi, w.rt_lo);
    NGB_LAUNCH_CHECK("cg_init_kernel");
    NGB_CUDA_TRY(cudaMemsetAsync(p1, 0, size_t(desc->nx) * desc->ny * desc->nz * sizeof(T), s));
    const int   grid_a = std::min(grid, pass_a_items(d)), grid_b = std::min(grid, pass_b_items(d));
    cudaEvent_t ev[3];
    for (auto& e : ev) NGB_CUDA_TRY(cudaEventCreate(&e));
    NGB_CUDA_TRY(cudaEventRecord(ev[0], s));
    for (int it = 0; it < reps; it++) {
        T* pa = (it % 2 == 0) ? p0 : p1;
        T* pb = (it % 2 == 0) ? p1 : p0;
        launch_pass_a<T>(d, grid_a, w.st, r, pa, pb, sv, w.partials, s);
    }
    NGB_CUDA_TRY(cudaEventRecord(ev[1], s));
    for (int it = 0; it < reps; it++) {
        T* pb = (it % 2 == 0) ? p1 : p0;
        if (d.bd)
            cg_pass_b_kernel<T, false><<<grid_b, kBX, 0, s>>>(d, w.st, xlo, pb, r, sv, w.partials, cudaGraphConditionalHandle{}, 0);
        else
            cg_pass_b_kernel<T, true><<<grid_b, kBX, 0, s>>>(d, w.st, xlo, pb, r, sv, w.partials, cudaGraphConditionalHandle{}, 0);
    }
    NGB_CUDA_TRY(cudaEventRecord(ev[2], s));
    NGB_LAUNCH_CHECK("cg_pass_a/b_kernel");
    NGB_CUDA_TRY(cudaEventSynchronize(ev[2]));
    float a = 0.f, bb = 0.f;
    NGB_CUDA_TRY(cudaEventElapsedTime(&a, ev[0], ev[1]));
    NGB_CUDA_TRY(cudaEventElapsedTime(&bb, ev[1], ev[2]));
    for (auto& e : ev) cudaEventDestroy(e);
    ms[0] = a / float(reps);
    ms[1] = bb / float(reps);
    return NGB_OK;
}

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_laplacian_apply(const ngb_poisson_desc* d, const void* u, void* out, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(u && out && u != out, "u/out must be distinct non-NULL device pointers");
    const Dom dom = make_dom(d);
    const int grid = grid_for(dom.segs);
    if (d->field == NGB_STORE_F64)
        laplacian_kernel<double><<<grid, kBX, 0, as_stream(stream)>>>(dom, static_cast<const double*>(u), static_cast<double*>(out));
    else
        laplacian_kernel<float><<<grid, kBX, 0, as_stream(stream)>>>(dom, static_cast<const float*>(u), static_cast<float*>(out));
    NGB_LAUNCH_CHECK("laplacian_kernel");
    return NGB_OK;
}

size_t ngb_dot_scratch_doubles(int64_t n)
{
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n + kBX - 1) / kBX, int64_t(sm_count()) * 4));
    return size_t(blocks) + 1;  // partials + one slot for the ticket
}

size_t ngb_fcg_scratch_doubles(int64_t n) { return 2 * (ngb_dot_scratch_doubles(n) - 1) + 1; }

int ngb_fcg_direction(int64_t n, void* z, void* az, const void* p_prev, const void* q_prev, const void* r, const double* zq,
                      const double* pq_prev, double* out, double* scratch, void* stream)
{
    NGB_CHECK_ARG(n > 0, "n must be positive");
    NGB_CHECK_ARG(z && az && r && out && scratch, "NULL argument");
    NGB_CHECK_ARG(!zq || (p_prev && q_prev && pq_prev), "zq given without p_prev, q_prev and pq_prev");
    cudaStream_t s = as_stream(stream);
    const int    blocks = int(ngb_dot_scratch_doubles(n) - 1);
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch + 2 * blocks);
    NGB_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
    fcg_direction_kernel<<<blocks, kBX, 0, s>>>(n, static_cast<float*>(z), static_cast<float*>(az), static_cast<const float*>(p_prev),
                                                static_cast<const float*>(q_prev), static_cast<const float*>(r), zq, pq_prev, out,
                                                scratch, ticket);
    NGB_LAUNCH_CHECK("fcg_direction_kernel");
    return NGB_OK;
}

int ngb_fcg_update(int64_t n, double* x, const void* p, void* r, const void* q, const double* pq_pr, double* rr, double* scratch,
                   void* stream)
{
    NGB_CHECK_ARG(n > 0, "n must be positive");
    NGB_CHECK_ARG(x && p && r && q && pq_pr && rr && scratch, "NULL argument");
    cudaStream_t s = as_stream(stream);
    const int    blocks = int(ngb_dot_scratch_doubles(n) - 1);
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch + 2 * blocks);
    NGB_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
    fcg_update_kernel<<<blocks, kBX, 0, s>>>(n, x, static_cast<const float*>(p), static_cast<float*>(r), static_cast<const float*>(q),
                                             pq_pr, rr, scratch, ticket);
    NGB_LAUNCH_CHECK("fcg_update_kernel");
    return NGB_OK;
}

int ngb_dot(int64_t n, int32_t field, const void* a, const void* b, double* result, double* scratch, void* stream)
{
    NGB_CHECK_ARG(n >= 0, "n < 0");
    NGB_CHECK_ARG(field == NGB_STORE_F32 || field == NGB_STORE_F64, "field must be F32 or F64");
    NGB_CHECK_ARG(result && scratch && (n == 0 || (a && b)), "NULL argument");
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        NGB_CUDA_TRY(cudaMemsetAsync(result, 0, sizeof(double), s));
        return NGB_OK;
    }
    const int     blocks = int(ngb_dot_scratch_doubles(n) - 1);
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch + blocks);
    NGB_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
    if (field == NGB_STORE_F64)
        dot_kernel<double><<<blocks, kBX, 0, s>>>(n, static_cast<const double*>(a), static_cast<const double*>(b), result, scratch,
                                                  ticket);
    else
        dot_kernel<float><<<blocks, kBX, 0, s>>>(n, static_cast<const float*>(a), static_cast<const float*>(b), result, scratch,
                                                 ticket);
    NGB_LAUNCH_CHECK("dot_kernel");
    return NGB_OK;
}

size_t ngb_cg_workspace_bytes(const ngb_poisson_desc* d)
{
    if (validate(d)) return 0;
    return layout(d, nullptr).bytes;
}

int ngb_cg_solve(const ngb_poisson_desc* d, const void* b, double* x, void* workspace, size_t workspace_bytes,
                 const ngb_cg_params* prm, ngb_cg_result* res, void* stream)
{
    NvtxRange nvtx("ngb_cg_solve");
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(b && x && workspace && prm, "NULL argument");
    NGB_CHECK_ARG(prm->refresh_every >= 1 && prm->check_every >= 1 && prm->max_iter >= 0, "bad CG params");
    NGB_CHECK_ARG(prm->tol >= 0, "tol < 0");
    NGB_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0, "workspace must be 256-byte aligned");
    const Workspace w = layout(d, workspace);
    NGB_CHECK_ARG(workspace_bytes >= w.bytes, "workspace too small (%zu < %zu)", workspace_bytes, w.bytes);
    NGB_CUDA_TRY(cudaMemsetAsync(&w.st->ticket, 0, sizeof(unsigned int), as_stream(stream)));
    if (d->field == NGB_STORE_F64) return solve_t<double>(d, static_cast<const double*>(b), x, w, prm, res, as_stream(stream));
    return solve_t<float>(d, static_cast<const float*>(b), x, w, prm, res, as_stream(stream));
}

int ngb_cg_time_passes(const ngb_poisson_desc* d, const void* b, double* x, void* workspace, size_t workspace_bytes,
                       int32_t reps, float* ms, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(b && x && workspace && ms && reps >= 1, "bad argument");
    NGB_CHECK_ARG((reinterpret_cast<uintptr_t>(workspace) & 255) == 0, "workspace must be 256-byte aligned");
    const Workspace w = layout(d, workspace);
    NGB_CHECK_ARG(workspace_bytes >= w.bytes, "workspace too small (%zu < %zu)", workspace_bytes, w.bytes);
    NGB_CUDA_TRY(cudaMemsetAsync(&w.st->ticket, 0, sizeof(unsigned int), as_stream(stream)));
    if (d->field == NGB_STORE_F64) return time_passes_t<double>(d, static_cast<const double*>(b), x, w, reps, ms, as_stream(stream));
    return time_passes_t<float>(d, static_cast<const float*>(b), x, w, reps, ms, as_stream(stream));
}

int ngb_poisson_rhs(const ngb_poisson_desc* d, const double* centres, const double* amps, double sigma, void* f, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(centres && amps && f && sigma > 0, "bad argument");
    const Dom dom = make_dom(d);
    rhs_kernel<<<grid_for(dom.segs), kBX, 0, as_stream(stream)>>>(dom, d->field, centres, amps, sigma, f);
    NGB_LAUNCH_CHECK("rhs_kernel");
    return NGB_OK;
}

int ngb_gaussian_sources(int32_t nx, int32_t ny, int32_t nz, uint64_t seed, double* centres, double* amps)
{
    NGB_CHECK_ARG(centres && amps && nx > 0 && ny > 0 && nz > 0, "bad argument");
    std::mt19937_64 g(seed);
    auto            u01 = [&]() { return double(g() >> 11) * (1.0 / 9007199254740992.0); };
    for (int k = 0; k < 8; k++) {
        centres[3 * k + 0] = nx / 8.0 + u01() * (0.75 * nx);
        centres[3 * k + 1] = ny / 8.0 + u01() * (0.75 * ny);
        centres[3 * k + 2] = nz / 8.0 + u01() * (0.75 * nz);
        amps[k] = 2.0 * u01() - 1.0;
    }
    return NGB_OK;
}

}  // extern "C"
