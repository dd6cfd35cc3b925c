// Checkpoint / resume of the dense LBM populations: a raw little-endian dump
// of one population buffer with a header that identifies the lattice (no
// reference counterpart: the reference writes VTK/VTI exports only,
// FieldBase.h:137, RunCavityTwoPop.cu:105-106). A resumed run continues bit
// for bit: the loader fills both ping-pong buffers with the saved state, so
// the wall nodes that no step writes match the original run's.
//
// File layout: "NGBLBM01", uint32 version (1), int32 nx, ny, nz, q, storage,
// int64 plane_stride, int64 step, double omega, uint64 payload bytes, then the
// payload (q * plane_stride elements of the storage type, the device image).
#include "common.cuh"
#include <cstring>

namespace ngb {
namespace {

struct CkptHeader {
    char     magic[8];
    uint32_t version;
    int32_t  nx, ny, nz, q, storage;
    int64_t  plane_stride, step;
    double   omega;
    uint64_t payload;
};
constexpr size_t kChunk = size_t(64) << 20;  // staging chunk (pinned)

int64_t stride_of(const ngb_lbm_dense_desc* d)
{
    return d->plane_stride > 0 ? d->plane_stride : int64_t(d->nx) * d->ny * d->nz;
}

int check_desc(const ngb_lbm_dense_desc* d)
{
    NGB_CHECK_ARG(d, "desc is NULL");
    NGB_CHECK_ARG(d->q == 19 || d->q == 27, "q must be 19 or 27");
    NGB_CHECK_ARG(d->storage >= NGB_STORE_F64 && d->storage <= NGB_STORE_F16SR, "unknown storage %d", d->storage);
    NGB_CHECK_ARG(d->nx > 0 && d->ny > 0 && d->nz > 0, "dims must be positive");
    return NGB_OK;
}

struct Pinned {
    void* p = nullptr;
    ~Pinned()
    {
        if (p) cudaFreeHost(p);
    }
};

struct File {
    FILE* f = nullptr;
    ~File()
    {
        if (f) std::fclose(f);
    }
};

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_lbm_dense_save(const char* path, const ngb_lbm_dense_desc* d, const void* f, int64_t step, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(path && f, "NULL argument");
    NvtxRange    nvtx("ngb_lbm_dense_save");
    cudaStream_t s = as_stream(stream);
    CkptHeader   h{};
    std::memcpy(h.magic, "NGBLBM01", 8);
    h.version = 1;
    h.nx = d->nx, h.ny = d->ny, h.nz = d->nz, h.q = d->q, h.storage = d->storage;
    h.plane_stride = stride_of(d);
    h.step = step;
    h.omega = d->omega;
    h.payload = uint64_t(d->q) * uint64_t(h.plane_stride) * storage_bytes(d->storage);
    Pinned buf;
    NGB_CUDA_TRY(cudaMallocHost(&buf.p, kChunk));
    File file;
    file.f = std::fopen(path, "wb");
    if (!file.f) {
        set_error("cannot open %s for writing", path);
        return NGB_ERR_INVALID;
    }
    if (std::fwrite(&h, sizeof(h), 1, file.f) != 1) {
        set_error("write of %s failed", path);
        return NGB_ERR_INVALID;
    }
    const char* src = static_cast<const char*>(f);
    for (uint64_t off = 0; off < h.payload; off += kChunk) {
        const size_t n = size_t(h.payload - off < kChunk ? h.payload - off : kChunk);
        NGB_CUDA_TRY(cudaMemcpyAsync(buf.p, src + off, n, cudaMemcpyDeviceToHost, s));
        NGB_CUDA_TRY(cudaStreamSynchronize(s));
        if (std::fwrite(buf.p, 1, n, file.f) != n) {
            set_error("write of %s failed", path);
            return NGB_ERR_INVALID;
        }
    }
    if (std::fclose(file.f) != 0) {
        file.f = nullptr;
        set_error("close of %s failed", path);
        return NGB_ERR_INVALID;
    }
    file.f = nullptr;
    return NGB_OK;
}

int ngb_lbm_dense_load(const char* path, const ngb_lbm_dense_desc* d, void* fa, void* fb, int64_t* step, void* stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    NGB_CHECK_ARG(path && fa, "NULL argument");
    NvtxRange    nvtx("ngb_lbm_dense_load");
    cudaStream_t s = as_stream(stream);
    File         file;
    file.f = std::fopen(path, "rb");
    if (!file.f) {
        set_error("cannot open %s", path);
        return NGB_ERR_INVALID;
    }
    CkptHeader h{};
    if (std::fread(&h, sizeof(h), 1, file.f) != 1 || std::memcmp(h.magic, "NGBLBM01", 8) != 0 || h.version != 1) {
        set_error("%s is not a population checkpoint of this library (NGBLBM01)", path);
        return NGB_ERR_INVALID;
    }
    if (h.nx != d->nx || h.ny != d->ny || h.nz != d->nz || h.q != d->q || h.storage != d->storage ||
        h.plane_stride != stride_of(d)) {
        set_error("checkpoint %s holds a %dx%dx%d D3Q%d lattice, storage %d, plane stride %lld; the desc asks for "
                  "%dx%dx%d D3Q%d, storage %d, plane stride %lld",
                  path, h.nx, h.ny, h.nz, h.q, h.storage, (long long)h.plane_stride, d->nx, d->ny, d->nz, d->q, d->storage,
                  (long long)stride_of(d));
        return NGB_ERR_INVALID;
    }
    const uint64_t payload = uint64_t(d->q) * uint64_t(h.plane_stride) * storage_bytes(d->storage);
    if (h.payload != payload) {
        set_error("checkpoint %s: payload of %llu bytes, expected %llu", path, (unsigned long long)h.payload,
                  (unsigned long long)payload);
        return NGB_ERR_INVALID;
    }
    Pinned buf;
    NGB_CUDA_TRY(cudaMallocHost(&buf.p, kChunk));
    char* dst = static_cast<char*>(fa);
    for (uint64_t off = 0; off < payload; off += kChunk) {
        const size_t n = size_t(payload - off < kChunk ? payload - off : kChunk);
        NGB_CUDA_TRY(cudaStreamSynchronize(s));  // the staging buffer is free again
        if (std::fread(buf.p, 1, n, file.f) != n) {
            set_error("checkpoint %s is truncated", path);
            return NGB_ERR_INVALID;
        }
        NGB_CUDA_TRY(cudaMemcpyAsync(dst + off, buf.p, n, cudaMemcpyHostToDevice, s));
    }
    if (fb) NGB_CUDA_TRY(cudaMemcpyAsync(fb, fa, size_t(payload), cudaMemcpyDeviceToDevice, s));
    NGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (step) *step = h.step;
    return NGB_OK;
}

}  // extern "C"
