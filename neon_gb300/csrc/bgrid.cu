// bGrid construction on the device, wall mask, flag scatter and the integer
// 6-neighbour known-answer operator.
#include "bgrid.cuh"

namespace ngb {
namespace {

// One warp per candidate block: the 16 mask words come from one ballot each
// (word w covers voxels 32w .. 32w+31 = lanes, bit = voxel & 31).
__device__ __forceinline__ uint32_t block_word(const uint8_t* __restrict__ active, int nx, int ny, int nz, int bx, int by, int bz,
                                               int w, int lane)
{
    const int v = 32 * w + lane;
    const int x = bx * 8 + (v & 7), y = by * 8 + ((v >> 3) & 7), z = bz * 8 + (v >> 6);
    bool      a = false;
    if (x < nx && y < ny && z < nz) a = __ldg(active + size_t(x) + size_t(nx) * (size_t(y) + size_t(ny) * z)) != 0;
    return __ballot_sync(0xffffffffu, a);
}

__global__ void bgrid_flag_kernel(const uint8_t* __restrict__ active, int nx, int ny, int nz, int bnx, int bny, int64_t ncand,
                                  int32_t* block_of)
{
    const int64_t cand = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
    const int     lane = threadIdx.x & 31;
    if (cand >= ncand) return;
    const int bx = int(cand % bnx), by = int((cand / bnx) % bny), bz = int(cand / (int64_t(bnx) * bny));
    uint32_t  any = 0;
    for (int w = 0; w < 16; w++) any |= block_word(active, nx, ny, nz, bx, by, bz, w, lane);
    if (lane == 0) block_of[cand] = any ? 1 : 0;
}

// Ranks of the active candidates (block_of[c] = rank or -1) by a three-kernel
// scan: per-tile counts of kScanTile candidates, an exclusive scan of the
// tile counts, and per-tile ranks from a CTA-wide scan plus the tile's
// offset. Every kernel is parallel over tiles except the scan of the tile
// counts (one per 4096 candidates).
constexpr int kScanThreads = 1024, kScanPer = 4, kScanTile = kScanThreads * kScanPer;

// Inclusive CTA-wide scan of one value per thread (warp shuffles, then the
// warp totals); returns the thread's inclusive prefix and the CTA total.
__device__ __forceinline__ uint32_t cta_scan(uint32_t v, uint32_t& total)
{
    __shared__ uint32_t warp_sum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warp_sum[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_sum[lane] = w;
    }
    __syncthreads();
    total = warp_sum[kScanThreads / 32 - 1];
    const uint32_t r = v + (warp > 0 ? warp_sum[warp - 1] : 0u);
    __syncthreads();  // warp_sum is reused by the next call
    return r;
}

__global__ void __launch_bounds__(kScanThreads) bgrid_tile_count_kernel(const int32_t* __restrict__ block_of, int64_t ncand,
                                                                       uint32_t* part)
{
    const int64_t c0 = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanPer;
    uint32_t      n = 0;
#pragma unroll
    for (int e = 0; e < kScanPer; e++) n += (c0 + e < ncand && block_of[c0 + e]) ? 1u : 0u;
    uint32_t total;
    cta_scan(n, total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// One CTA: part[i] <- sum of part[0 .. i-1]; *n_blocks = sum of all.
__global__ void __launch_bounds__(kScanThreads) bgrid_part_scan_kernel(uint32_t* part, int64_t nparts, uint32_t* n_blocks)
{
    uint32_t carry = 0;
    for (int64_t base = 0; base < nparts; base += kScanThreads) {
        const int64_t i = base + threadIdx.x;
        const uint32_t v = i < nparts ? part[i] : 0u;
        uint32_t       total;
        const uint32_t incl = cta_scan(v, total);
        if (i < nparts) part[i] = carry + incl - v;
        carry += total;
    }
    if (threadIdx.x == 0) *n_blocks = carry;
}

__global__ void __launch_bounds__(kScanThreads) bgrid_tile_rank_kernel(int32_t* block_of, int64_t ncand, const uint32_t* part)
{
    const int64_t c0 = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanPer;
    int32_t       f[kScanPer];
    uint32_t      n = 0;
#pragma unroll
    for (int e = 0; e < kScanPer; e++) {
        f[e] = c0 + e < ncand ? block_of[c0 + e] : 0;
        n += f[e] ? 1u : 0u;
    }
    uint32_t       total;
    uint32_t       run = part[blockIdx.x] + cta_scan(n, total) - n;
#pragma unroll
    for (int e = 0; e < kScanPer; e++)
        if (c0 + e < ncand) block_of[c0 + e] = f[e] ? int32_t(run++) : -1;
}

__global__ void bgrid_fill_kernel(const uint8_t* __restrict__ active, int nx, int ny, int nz, int bnx, int bny, int bnz,
                                  const int32_t* __restrict__ block_of, int32_t* origin, uint32_t* mask, uint32_t* conn,
                                  unsigned long long* n_active)
{
    const int64_t ncand = int64_t(bnx) * bny * bnz;
    const int64_t cand = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
    const int     lane = threadIdx.x & 31;
    if (cand >= ncand) return;
    const int32_t b = block_of[cand];
    if (b < 0) return;
    const int bx = int(cand % bnx), by = int((cand / bnx) % bny), bz = int(cand / (int64_t(bnx) * bny));
    uint32_t  count = 0, mine = 0;
    for (int w = 0; w < 16; w++) {
        const uint32_t word = block_word(active, nx, ny, nz, bx, by, bz, w, lane);
        count += __popc(word);
        if (lane == w) mine = word;
    }
    if (lane < 16) mask[size_t(b) * 16 + lane] = mine;
    if (lane < 3) origin[size_t(b) * 3 + lane] = 8 * (lane == 0 ? bx : (lane == 1 ? by : bz));
    if (lane < 27) {
        const int i = lane % 3, j = (lane / 3) % 3, k = lane / 9;
        const int nbx = bx + i - 1, nby = by + j - 1, nbz = bz + k - 1;
        uint32_t  v = NGB_BGRID_NO_BLOCK;
        if (nbx >= 0 && nby >= 0 && nbz >= 0 && nbx < bnx && nby < bny && nbz < bnz) {
            const int32_t id = block_of[nbx + int64_t(bnx) * (nby + int64_t(bny) * nbz)];
            if (id >= 0) v = uint32_t(id);
        }
        conn[size_t(b) * 27 + lane] = v;
    }
    if (lane == 0 && n_active) atomicAdd(n_active, (unsigned long long)count);
}

template <int Q>
__global__ void bgrid_wall_mask_kernel(const uint32_t* __restrict__ mask, const uint32_t* __restrict__ conn, uint32_t* flags)
{
    const uint32_t b = blockIdx.x;
    const int      v = threadIdx.x, i = v & 7, j = (v >> 3) & 7, k = v >> 6;
    const size_t   cell = size_t(b) * kBlockVoxels + v;
    const uint32_t f = flags[cell];
    if (flag_class(f) != NGB_CELL_BULK) {
        flags[cell] = make_flag(0, flag_class(f));
        return;
    }
    uint32_t m = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int cx = Lattice<Q>::cx(q), cy = Lattice<Q>::cy(q), cz = Lattice<Q>::cz(q);
        if (cx == 0 && cy == 0 && cz == 0) continue;
        uint32_t nb;
        int      nv;
        bool     wall = true;
        if (bgrid_valid_ngh(mask, conn, b, i, j, k, -cx, -cy, -cz, nb, nv))
            wall = !is_fluid_class(flag_class(flags[size_t(nb) * kBlockVoxels + nv]));
        if (wall) m |= 1u << q;
    }
    flags[cell] = make_flag(m, NGB_CELL_BULK);
}

__global__ void bgrid_flags_from_dense_kernel(const int32_t* __restrict__ origin, const uint32_t* __restrict__ mask, int nx, int ny,
                                              int nz, const uint8_t* __restrict__ cls, uint32_t* flags)
{
    const uint32_t b = blockIdx.x;
    const int      v = threadIdx.x;
    const int      x = origin[3 * b] + (v & 7), y = origin[3 * b + 1] + ((v >> 3) & 7), z = origin[3 * b + 2] + (v >> 6);
    int            c = NGB_CELL_UNDEFINED;
    if (x < nx && y < ny && z < nz && bgrid_active(mask, b, v)) c = cls[size_t(x) + size_t(nx) * (size_t(y) + size_t(ny) * z)];
    flags[size_t(b) * kBlockVoxels + v] = make_flag(0, c);
}

__global__ void bgrid_laplace_i64_kernel(const uint32_t* __restrict__ mask, const uint32_t* __restrict__ conn,
                                         const int64_t* __restrict__ a, int64_t* __restrict__ out)
{
    const uint32_t b = blockIdx.x;
    const int      v = threadIdx.x, i = v & 7, j = (v >> 3) & 7, k = v >> 6;
    if (!bgrid_active(mask, b, v)) return;
    const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    int64_t   sum = 0;
    int       count = 0;
#pragma unroll
    for (int d = 0; d < 6; d++) {
        uint32_t nb;
        int      nv;
        if (bgrid_valid_ngh(mask, conn, b, i, j, k, off[d][0], off[d][1], off[d][2], nb, nv)) {
            sum += a[size_t(nb) * kBlockVoxels + nv];
            count++;
        }
    }
    const size_t cell = size_t(b) * kBlockVoxels + v;
    out[cell] = a[cell] - int64_t(count) * sum;
}

__global__ void dense_laplace_i64_kernel(int nx, int ny, int nz, const int64_t* __restrict__ a, int64_t* __restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= nx) return;
    const int64_t sy = nx, sz = int64_t(nx) * ny, cell = x + sy * y + sz * z;
    int64_t       sum = 0;
    int           count = 0;
    if (x + 1 < nx) sum += a[cell + 1], count++;
    if (x > 0) sum += a[cell - 1], count++;
    if (y + 1 < ny) sum += a[cell + sy], count++;
    if (y > 0) sum += a[cell - sy], count++;
    if (z + 1 < nz) sum += a[cell + sz], count++;
    if (z > 0) sum += a[cell - sz], count++;
    out[cell] = a[cell] - int64_t(count) * sum;
}

int validate_bgrid(const ngb_bgrid_desc* d)
{
    NGB_CHECK_ARG(d, "desc is NULL");
    NGB_CHECK_ARG(d->n_blocks >= 0, "n_blocks < 0");
    NGB_CHECK_ARG(d->q == 19 || d->q == 27, "q must be 19 or 27 (got %d)", d->q);
    NGB_CHECK_ARG(d->storage >= NGB_STORE_F64 && d->storage <= NGB_STORE_BF16OFF, "bad storage %d", d->storage);
    NGB_CHECK_ARG(d->n_blocks == 0 || (d->origin && d->mask && d->conn), "bGrid arrays must be non-NULL");
    return NGB_OK;
}

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_bgrid_count(int32_t nx, int32_t ny, int32_t nz, const uint8_t* active, int32_t* block_of, uint32_t* n_blocks,
                    void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "dims must be positive");
    NGB_CHECK_ARG(active && block_of && n_blocks, "NULL argument");
    const int     bnx = NGB_BGRID_BLOCKS(nx), bny = NGB_BGRID_BLOCKS(ny), bnz = NGB_BGRID_BLOCKS(nz);
    const int64_t ncand = int64_t(bnx) * bny * bnz;
    NGB_CHECK_ARG(ncand < (int64_t(1) << 31), "too many candidate blocks");
    cudaStream_t  s = as_stream(stream);
    const int     threads = 256;
    const int64_t blocks = (ncand * 32 + threads - 1) / threads;
    bgrid_flag_kernel<<<dim3(unsigned(blocks)), threads, 0, s>>>(active, nx, ny, nz, bnx, bny, ncand, block_of);
    NGB_LAUNCH_CHECK("bgrid_flag_kernel");
    const int64_t nparts = (ncand + kScanTile - 1) / kScanTile;
    uint32_t*     part = nullptr;  // per-tile counts, stream-ordered scratch
    NGB_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&part), size_t(nparts) * sizeof(uint32_t), s));
    bgrid_tile_count_kernel<<<unsigned(nparts), kScanThreads, 0, s>>>(block_of, ncand, part);
    bgrid_part_scan_kernel<<<1, kScanThreads, 0, s>>>(part, nparts, n_blocks);
    bgrid_tile_rank_kernel<<<unsigned(nparts), kScanThreads, 0, s>>>(block_of, ncand, part);
    const cudaError_t e = cudaGetLastError();
    cudaFreeAsync(part, s);
    if (e != cudaSuccess) {
        set_error("bGrid block scan failed: %s", cudaGetErrorString(e));
        return NGB_ERR_CUDA;
    }
    return NGB_OK;
}

int ngb_bgrid_fill(int32_t nx, int32_t ny, int32_t nz, const uint8_t* active, const int32_t* block_of, int32_t* origin,
                   uint32_t* mask, uint32_t* conn, unsigned long long* n_active_voxels, void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0, "dims must be positive");
    NGB_CHECK_ARG(active && block_of && origin && mask && conn, "NULL argument");
    const int     bnx = NGB_BGRID_BLOCKS(nx), bny = NGB_BGRID_BLOCKS(ny), bnz = NGB_BGRID_BLOCKS(nz);
    const int64_t ncand = int64_t(bnx) * bny * bnz;
    cudaStream_t  s = as_stream(stream);
    if (n_active_voxels) NGB_CUDA_TRY(cudaMemsetAsync(n_active_voxels, 0, sizeof(unsigned long long), s));
    const int     threads = 256;
    const int64_t blocks = (ncand * 32 + threads - 1) / threads;
    bgrid_fill_kernel<<<dim3(unsigned(blocks)), threads, 0, s>>>(active, nx, ny, nz, bnx, bny, bnz, block_of, origin, mask, conn,
                                                               n_active_voxels);
    NGB_LAUNCH_CHECK("bgrid_fill_kernel");
    return NGB_OK;
}

int ngb_bgrid_wall_mask(const ngb_bgrid_desc* d, uint32_t* flags, void* stream)
{
    int rc = validate_bgrid(d);
    if (rc) return rc;
    NGB_CHECK_ARG(flags, "flags is NULL");
    if (d->n_blocks == 0) return NGB_OK;
    if (d->q == 19)
        bgrid_wall_mask_kernel<19><<<d->n_blocks, kBlockVoxels, 0, as_stream(stream)>>>(d->mask, d->conn, flags);
    else
        bgrid_wall_mask_kernel<27><<<d->n_blocks, kBlockVoxels, 0, as_stream(stream)>>>(d->mask, d->conn, flags);
    NGB_LAUNCH_CHECK("bgrid_wall_mask_kernel");
    return NGB_OK;
}

int ngb_bgrid_flags_from_dense(const ngb_bgrid_desc* d, int32_t nx, int32_t ny, int32_t nz, const uint8_t* cls, uint32_t* flags,
                               void* stream)
{
    int rc = validate_bgrid(d);
    if (rc) return rc;
    NGB_CHECK_ARG(cls && flags && nx > 0 && ny > 0 && nz > 0, "bad argument");
    if (d->n_blocks == 0) return NGB_OK;
    bgrid_flags_from_dense_kernel<<<d->n_blocks, kBlockVoxels, 0, as_stream(stream)>>>(d->origin, d->mask, nx, ny, nz, cls, flags);
    NGB_LAUNCH_CHECK("bgrid_flags_from_dense_kernel");
    return NGB_OK;
}

int ngb_bgrid_laplace_i64(const ngb_bgrid_desc* d, const int64_t* a, int64_t* b, void* stream)
{
    NGB_CHECK_ARG(d && d->n_blocks >= 0 && (d->n_blocks == 0 || (d->mask && d->conn)), "bad bGrid desc");
    NGB_CHECK_ARG(a && b && a != b, "a/b must be distinct non-NULL");
    if (d->n_blocks == 0) return NGB_OK;
    bgrid_laplace_i64_kernel<<<d->n_blocks, kBlockVoxels, 0, as_stream(stream)>>>(d->mask, d->conn, a, b);
    NGB_LAUNCH_CHECK("bgrid_laplace_i64_kernel");
    return NGB_OK;
}

int ngb_dense_laplace_i64(int32_t nx, int32_t ny, int32_t nz, const int64_t* a, int64_t* b, void* stream)
{
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0 && ny <= 65535 && nz <= 65535, "bad dims");
    NGB_CHECK_ARG(a && b && a != b, "a/b must be distinct non-NULL");
    dense_laplace_i64_kernel<<<dim3((nx + 127) / 128, ny, nz), 128, 0, as_stream(stream)>>>(nx, ny, nz, a, b);
    NGB_LAUNCH_CHECK("dense_laplace_i64_kernel");
    return NGB_OK;
}

}  // extern "C"
