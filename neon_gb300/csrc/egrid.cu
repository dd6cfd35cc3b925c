// eGrid (element-sparse grid) construction on the device, one partition.
//
// Neon builds an eGrid with the block partitioner at block size 1
// (eGrid_imp.h:8-129 -> Partitioner1D): on one partition every active cell is
// an internal element, in the scan order z, then y, then x fastest
// (SpanClassifier.h:228-237), its global position is the cell itself
// (Partitioner1D.h:212-255) and its connectivity holds, per stencil point s,
// the element at position + offset_s or "no neighbour" (Partitioner1D.h:338-
// 380), read as conn[s * count + e] with a negative value meaning invalid
// (ePartition_imp.h isValidNgh).
//
// count: a chunked scan of the active map (per-chunk totals, one CTA scanning
// the totals, per-chunk ranks with warp ballots) gives every cell its element
// index or -1. fill: origins from the index map, then one thread per element
// looks up its stencil neighbours in the index map.
#include "common.cuh"

namespace ngb {
namespace {

constexpr int kEChunk = 2048;  // cells per CTA of the scan (256 threads x 8)
constexpr int kEThreads = 256;
constexpr int kEMaxPoints = 64;

struct EPoints {
    int8_t x[kEMaxPoints], y[kEMaxPoints], z[kEMaxPoints];
    int    n;
};

__global__ void __launch_bounds__(kEThreads) egrid_chunk_kernel(const uint8_t* __restrict__ active, int64_t V, int32_t* chunk_sum)
{
    __shared__ int warp_sum[kEThreads / 32];
    const int64_t  c0 = int64_t(blockIdx.x) * kEChunk;
    int            local = 0;
#pragma unroll
    for (int k = 0; k < kEChunk / kEThreads; k++) {
        const int64_t i = c0 + k * kEThreads + threadIdx.x;
        local += (i < V && __ldg(active + i)) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kEThreads / 32; w++) t += warp_sum[w];
        chunk_sum[blockIdx.x] = t;
    }
}

// Exclusive scan of the chunk totals in place (one CTA); *count = the total.
constexpr int kEScanThreads = 1024;
__global__ void __launch_bounds__(kEScanThreads) egrid_scan_kernel(int32_t* chunk_sum, int64_t nchunks, int32_t* count)
{
    __shared__ int32_t part[kEScanThreads];
    const int64_t      per = (nchunks + kEScanThreads - 1) / kEScanThreads;
    const int64_t      b0 = threadIdx.x * per, b1 = min(nchunks, b0 + per);
    int32_t            local = 0;
    for (int64_t c = b0; c < b1; c++) local += chunk_sum[c];
    part[threadIdx.x] = local;
    __syncthreads();
    for (int off = 1; off < kEScanThreads; off <<= 1) {
        const int32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int32_t run = part[threadIdx.x] - local;
    for (int64_t c = b0; c < b1; c++) {
        const int32_t v = chunk_sum[c];
        chunk_sum[c] = run;
        run += v;
    }
    if (threadIdx.x == kEScanThreads - 1) *count = part[kEScanThreads - 1];
}

// Element index of every cell of the chunk (scan order), -1 when inactive.
__global__ void __launch_bounds__(kEThreads) egrid_rank_kernel(const uint8_t* __restrict__ active, int64_t V,
                                                               const int32_t* __restrict__ chunk_base, int32_t* elem_of)
{
    __shared__ int warp_tot[kEThreads / 32];
    const int64_t  c0 = int64_t(blockIdx.x) * kEChunk;
    const int      lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    int32_t        base = chunk_base[blockIdx.x];
    for (int k = 0; k < kEChunk / kEThreads; k++) {
        const int64_t  i = c0 + k * kEThreads + threadIdx.x;
        const bool     a = i < V && __ldg(active + i);
        const uint32_t bal = __ballot_sync(0xffffffffu, a);
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        int off = 0, tot = 0;
        for (int w = 0; w < kEThreads / 32; w++) {
            off += w < warp ? warp_tot[w] : 0;
            tot += warp_tot[w];
        }
        if (i < V) elem_of[i] = a ? base + off + __popc(bal & lt) : -1;
        base += tot;
        __syncthreads();
    }
}

__global__ void egrid_origin_kernel(int nx, int ny, int64_t V, const int32_t* __restrict__ elem_of, int32_t* origin)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const int32_t e = elem_of[i];
    if (e < 0) return;
    origin[3 * int64_t(e)] = int32_t(i % nx);
    origin[3 * int64_t(e) + 1] = int32_t((i / nx) % ny);
    origin[3 * int64_t(e) + 2] = int32_t(i / (int64_t(nx) * ny));
}

__global__ void egrid_conn_kernel(int nx, int ny, int nz, const int32_t* __restrict__ elem_of, const int32_t* __restrict__ origin,
                                  int32_t count, const EPoints pts, int32_t* conn)
{
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const int x = origin[3 * e], y = origin[3 * e + 1], z = origin[3 * e + 2];
    for (int s = 0; s < pts.n; s++) {
        const int xx = x + pts.x[s], yy = y + pts.y[s], zz = z + pts.z[s];
        int32_t   v = -1;
        if (xx >= 0 && yy >= 0 && zz >= 0 && xx < nx && yy < ny && zz < nz)
            v = elem_of[int64_t(xx) + int64_t(nx) * (int64_t(yy) + int64_t(ny) * zz)];
        conn[int64_t(s) * count + e] = v;
    }
}

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_egrid_count(int32_t nx, int32_t ny, int32_t nz, const uint8_t* active, int32_t* elem_of, int32_t* scratch, int32_t* count,
                    void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "dims must be positive");
    NGB_CHECK_ARG(active && elem_of && scratch && count, "NULL argument");
    const int64_t V = int64_t(nx) * ny * nz;
    NGB_CHECK_ARG(V < (int64_t(1) << 31), "an eGrid holds fewer than 2^31 cells");
    const int64_t nchunks = (V + kEChunk - 1) / kEChunk;
    cudaStream_t  s = as_stream(stream);
    egrid_chunk_kernel<<<unsigned(nchunks), kEThreads, 0, s>>>(active, V, scratch);
    NGB_LAUNCH_CHECK("egrid_chunk_kernel");
    egrid_scan_kernel<<<1, kEScanThreads, 0, s>>>(scratch, nchunks, count);
    NGB_LAUNCH_CHECK("egrid_scan_kernel");
    egrid_rank_kernel<<<unsigned(nchunks), kEThreads, 0, s>>>(active, V, scratch, elem_of);
    NGB_LAUNCH_CHECK("egrid_rank_kernel");
    return NGB_OK;
}

int ngb_egrid_fill(int32_t nx, int32_t ny, int32_t nz, const int32_t* elem_of, int32_t count, const int8_t* points, int32_t npts,
                   int32_t* origin, int32_t* conn, void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "dims must be positive");
    NGB_CHECK_ARG(count >= 0, "count < 0");
    NGB_CHECK_ARG(npts >= 0 && npts <= kEMaxPoints, "at most %d stencil points (got %d)", kEMaxPoints, npts);
    NGB_CHECK_ARG(elem_of && origin && (npts == 0 || (points && conn)), "NULL argument");
    const int64_t V = int64_t(nx) * ny * nz;
    NGB_CHECK_ARG(V < (int64_t(1) << 31), "an eGrid holds fewer than 2^31 cells");
    EPoints p{};
    p.n = npts;
    for (int s = 0; s < npts; s++) {
        p.x[s] = points[3 * s], p.y[s] = points[3 * s + 1], p.z[s] = points[3 * s + 2];
        NGB_CHECK_ARG(p.x[s] >= -64 && p.x[s] <= 64 && p.y[s] >= -64 && p.y[s] <= 64 && p.z[s] >= -64 && p.z[s] <= 64,
                      "stencil offsets out of range");
    }
    cudaStream_t s = as_stream(stream);
    egrid_origin_kernel<<<unsigned((V + 255) / 256), 256, 0, s>>>(nx, ny, V, elem_of, origin);
    NGB_LAUNCH_CHECK("egrid_origin_kernel");
    if (count > 0 && npts > 0) {
        egrid_conn_kernel<<<unsigned((count + 255) / 256), 256, 0, s>>>(nx, ny, nz, elem_of, origin, count, p, conn);
        NGB_LAUNCH_CHECK("egrid_conn_kernel");
    }
    return NGB_OK;
}

}  // extern "C"
