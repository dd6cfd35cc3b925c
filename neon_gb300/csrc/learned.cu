// Learned-preconditioner Poisson solver behind the C ABI: flexible CG (FCG(1))
// whose preconditioner is a V-cycle (damped-Jacobi smoothing, full-weighting
// restriction, trilinear prolongation) with the U-Net as the coarsest-level
// solve, the true residual b - A x recomputed in FP64, and Jacobi-PCG
// (ngb_cg_solve) as the fallback on stagnation or breakdown. No reference
// counterpart: libNeonSolver offers plain CG only
// (libNeonSolver/include/Neon/solver/linear/krylov/CG.h:70-76); the solver is
// its learned sibling with the same solve(b, x) -> result shape.
//
// The solver owns its device buffers (created once per grid size, like a
// Neon solver owns its fields) and calls only this library's kernels:
//   network: ngb_unet_input, ngb_conv3d_tc / ngb_conv3d, ngb_pool2, ngb_up2,
//            ngb_unet_output (3-level U-Net 16/32/64, BF16 activations);
//   V-cycle: ngb_mg_jacobi, ngb_mg_residual, ngb_mg_restrict,
//            ngb_mg_prolong_add, ngb_mg_apply, ngb_dot, ngb_scale_by_ratio;
//   FCG:     ngb_fcg_direction, ngb_fcg_update, ngb_dot, and the fused FP64
//            true-residual kernel below.
// The host reads one double per iteration (|r|^2 for the stopping test).
#include "common.cuh"
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

namespace ngb {
namespace {

struct LayerShape {
    int cin, cout, level;
};
// Layer order of the weight file and of the network (bias-free, ReLU after every
// convolution but the last): level 0 = the grid the network runs on.
constexpr LayerShape kLayers[10] = {{16, 16, 0}, {16, 16, 0}, {16, 32, 1}, {32, 32, 1}, {32, 64, 2},
                                    {64, 64, 2}, {96, 32, 1}, {32, 32, 1}, {48, 16, 0}, {16, 16, 0}};
constexpr int kNumLayers = 10;

int64_t layer_count(int l) { return int64_t(kLayers[l].cout) * 27 * kLayers[l].cin; }
int64_t total_count()
{
    int64_t c = 0;
    for (int l = 0; l < kNumLayers; l++) c += layer_count(l);
    return c;
}

// FP32 -> BF16 round-to-nearest-even (the rounding of torch's .to(bfloat16)).
uint16_t bf16_rne(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    if ((x & 0x7fffffffu) > 0x7f800000u) return uint16_t((x >> 16) | 0x40u);
    x += 0x7fffu + ((x >> 16) & 1u);
    return uint16_t(x >> 16);
}
float bf16_to_f32(uint16_t h)
{
    const uint32_t x = uint32_t(h) << 16;
    float          f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ---------------------------------------------------------------- fused FP64 true residual
// r = float(b - A x) on interior nodes (A: 7-point operator with spacing h),
// 0 on the box faces; partial[block] = sum of (b - A x)^2 over the block's
// nodes (FP64). finalize sums the partials in block order (deterministic).
constexpr int kResThreads = 256;

__global__ void __launch_bounds__(kResThreads) true_residual_kernel(int n, double invh2, const float* __restrict__ b,
                                                                    const double* __restrict__ x, float* __restrict__ r,
                                                                    double* __restrict__ partial)
{
    __shared__ double red[kResThreads];
    const int64_t     V = int64_t(n) * n * n, sy = n, sz = int64_t(n) * n;
    double            acc = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * kResThreads + threadIdx.x; i < V; i += int64_t(gridDim.x) * kResThreads) {
        const int xx = int(i % n), yy = int((i / n) % n), zz = int(i / sz);
        float     rv = 0.f;
        if (xx > 0 && yy > 0 && zz > 0 && xx < n - 1 && yy < n - 1 && zz < n - 1) {
            const double s = x[i - 1] + x[i + 1] + x[i - sy] + x[i + sy] + x[i - sz] + x[i + sz];
            const double rt = double(b[i]) - (6.0 * x[i] - s) * invh2;
            rv = float(rt);
            acc += rt * rt;
        }
        r[i] = rv;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kResThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(kResThreads) sum_partials_kernel(int m, const double* __restrict__ partial, double* out)
{
    __shared__ double red[kResThreads];
    double            s = 0.0;
    for (int i = threadIdx.x; i < m; i += kResThreads) s += partial[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kResThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

ngb_poisson_desc box_desc(int n, int field, double h)
{
    ngb_poisson_desc d{};
    d.nx = d.ny = d.nz = n;
    d.field = field;
    d.h = h;
    d.bd = nullptr;
    return d;
}

#define NGB_TRY(expr)               \
    do {                            \
        const int rc_ = (expr);     \
        if (rc_ != NGB_OK) return rc_; \
    } while (0)

}  // namespace
}  // namespace ngb

using namespace ngb;

// ---------------------------------------------------------------- the solver object
struct ngb_learned_solver {
    int n = 0, levels = 0, nc = 0;  // fine size, V-cycle levels, coarsest size (the network's grid)
    bool net = true;                 // false: the same cycle without the coarsest correction
    double omega = 6.0 / 7.0;
    int    post = 2;
    std::vector<void*> allocs;
    // network
    void *in0 = nullptr, *a0 = nullptr, *cat0 = nullptr, *d0a = nullptr, *p0 = nullptr, *a1 = nullptr, *cat1 = nullptr,
         *d1a = nullptr, *d1b = nullptr, *p1 = nullptr, *a2 = nullptr, *b2 = nullptr;
    float* out = nullptr;
    void*  wb[kNumLayers] = {};  // BF16 [cout][27][cin]
    void*  wp[kNumLayers] = {};  // tensor-core operand image
    // V-cycle, per level
    std::vector<float*>           u, tmp, res, r;  // r[0] unused (the cycle's input)
    std::vector<ngb_poisson_desc> desc;
    float *e_c = nullptr, *ae_c = nullptr;
    double* scal_c = nullptr;  // |r|^2, <e, r>, <e, A e> of the coarse solve
    double* scratch_c = nullptr;
    // FCG
    float * r_f = nullptr, *z[2] = {nullptr, nullptr}, *az[2] = {nullptr, nullptr};
    double* scal = nullptr;  // zq, rr, (pq, pr) x 2
    double* scratch_fcg = nullptr;
    double* scratch_dot = nullptr;
    double* dotres = nullptr;
    double* partial = nullptr;
    int     res_blocks = 0;
    double* host = nullptr;  // pinned landing slot of the per-iteration read
    void*   cg_ws = nullptr;
    size_t  cg_ws_bytes = 0;

    ~ngb_learned_solver()
    {
        for (void* p : allocs) cudaFree(p);
        if (host) cudaFreeHost(host);
    }
    template <typename T>
    int alloc(T** p, size_t bytes)
    {
        void* q = nullptr;
        NGB_CUDA_TRY(cudaMalloc(&q, bytes));
        NGB_CUDA_TRY(cudaMemset(q, 0, bytes));
        allocs.push_back(q);
        *p = static_cast<T*>(q);
        return NGB_OK;
    }

    // ------------------------------------------------------------ network at nc^3
    int conv(int lvl, const void* x, int ldx, int xoff, int cin, int layer, void* y, int ldy, int yoff, int cout, bool out_f32,
             bool relu, cudaStream_t s)
    {
        const int   m = nc >> lvl;
        const char* xp = static_cast<const char*>(x) + size_t(xoff) * 2;
        char*       yp = static_cast<char*>(y) + size_t(yoff) * (out_f32 ? 4 : 2);
        if (ngb_conv3d_tc_supported(m, m, m, ldx, cin, ldy, cout))
            return ngb_conv3d_tc(m, m, m, xp, ldx, cin, wp[layer], nullptr, yp, ldy, cout, out_f32, relu, 0, s);
        for (int lo = 0; lo < cout; lo += 64) {  // the mma.sync kernel takes at most 64 output channels
            const int   hi = lo + 64 < cout ? lo + 64 : cout;
            const char* w = static_cast<const char*>(wb[layer]) + size_t(lo) * 27 * cin * 2;
            NGB_TRY(ngb_conv3d(m, m, m, xp, ldx, cin, w, nullptr, yp + size_t(lo) * (out_f32 ? 4 : 2), ldy, hi - lo, out_f32,
                               relu, 0, s));
        }
        return NGB_OK;
    }
    // e = scale * M(r) on the nc^3 grid, 0 on its faces; rr receives |r|^2.
    int network(const float* rin, float* e, double scale, double* rr, cudaStream_t s)
    {
        const int64_t V0 = int64_t(nc) * nc * nc;
        const int     m1 = nc >> 1;
        NGB_TRY(ngb_dot(V0, NGB_STORE_F32, rin, rin, rr, scratch_c, s));
        NGB_TRY(ngb_unet_input(V0, rin, rr, in0, 16, s));
        NGB_TRY(conv(0, in0, 16, 0, 16, 0, a0, 16, 0, 16, false, true, s));
        NGB_TRY(conv(0, a0, 16, 0, 16, 1, cat0, 48, 32, 16, false, true, s));
        NGB_TRY(ngb_pool2(nc, nc, nc, 16, static_cast<char*>(cat0) + 32 * 2, 48, p0, 16, s));
        NGB_TRY(conv(1, p0, 16, 0, 16, 2, a1, 32, 0, 32, false, true, s));
        NGB_TRY(conv(1, a1, 32, 0, 32, 3, cat1, 96, 64, 32, false, true, s));
        NGB_TRY(ngb_pool2(m1, m1, m1, 32, static_cast<char*>(cat1) + 64 * 2, 96, p1, 32, s));
        NGB_TRY(conv(2, p1, 32, 0, 32, 4, a2, 64, 0, 64, false, true, s));
        NGB_TRY(conv(2, a2, 64, 0, 64, 5, b2, 64, 0, 64, false, true, s));
        NGB_TRY(ngb_up2(m1, m1, m1, 64, b2, 64, cat1, 96, s));
        NGB_TRY(conv(1, cat1, 96, 0, 96, 6, d1a, 32, 0, 32, false, true, s));
        NGB_TRY(conv(1, d1a, 32, 0, 32, 7, d1b, 32, 0, 32, false, true, s));
        NGB_TRY(ngb_up2(nc, nc, nc, 32, d1b, 32, cat0, 48, s));
        NGB_TRY(conv(0, cat0, 48, 0, 48, 8, d0a, 16, 0, 16, false, true, s));
        NGB_TRY(conv(0, d0a, 16, 0, 16, 9, out, 16, 0, 16, true, false, s));
        return ngb_unet_output(nc, nc, nc, out, 16, rr, scale, e, s);
    }

    // ------------------------------------------------------------ V-cycle
    // Coarsest level: e = beta 4^L M(r_L), beta = <e, r> / <e, A e> (0 if e is
    // no descent direction).
    int coarse(const float* rl, cudaStream_t s)
    {
        const int64_t V = int64_t(nc) * nc * nc;
        NGB_TRY(network(rl, e_c, std::ldexp(1.0, 2 * levels), scal_c, s));
        NGB_TRY(ngb_mg_apply(&desc[levels], e_c, ae_c, s));
        NGB_TRY(ngb_dot(V, NGB_STORE_F32, e_c, rl, scal_c + 1, scratch_c, s));
        NGB_TRY(ngb_dot(V, NGB_STORE_F32, e_c, ae_c, scal_c + 2, scratch_c, s));
        return ngb_scale_by_ratio(V, e_c, scal_c + 1, scal_c + 2, s);
    }
    int cycle(int l, const float* rl, float* outl, cudaStream_t s)
    {
        if (l == levels) return coarse(rl, s);
        const ngb_poisson_desc* d = &desc[l];
        float*                  ul = outl ? outl : u[l];
        NGB_TRY(ngb_mg_jacobi(d, nullptr, rl, ul, omega, s));
        // without the network the level above the coarsest gets no correction
        if (net || l + 1 < levels) {
            NGB_TRY(ngb_mg_residual(d, ul, rl, res[l], s));
            NGB_TRY(ngb_mg_restrict(d, res[l], r[l + 1], 1.0, s));
            NGB_TRY(cycle(l + 1, r[l + 1], nullptr, s));
            NGB_TRY(ngb_mg_prolong_add(d, l + 1 == levels ? e_c : u[l + 1], ul, s));
        }
        float* a = ul;
        float* b = tmp[l];
        for (int k = 0; k < post; k++) {
            NGB_TRY(ngb_mg_jacobi(d, a, rl, b, omega, s));
            float* t = a;
            a = b;
            b = t;
        }
        if (a != ul) NGB_CUDA_TRY(cudaMemcpyAsync(ul, a, size_t(d->nx) * d->ny * d->nz * 4, cudaMemcpyDeviceToDevice, s));
        return NGB_OK;
    }

    // ------------------------------------------------------------ FCG
    int true_residual(const float* b, const double* x, double bn, double* rel, cudaStream_t s)
    {
        true_residual_kernel<<<res_blocks, kResThreads, 0, s>>>(n, 1.0, b, x, r_f, partial);
        NGB_LAUNCH_CHECK("true_residual_kernel");
        sum_partials_kernel<<<1, kResThreads, 0, s>>>(res_blocks, partial, dotres);
        NGB_LAUNCH_CHECK("sum_partials_kernel");
        NGB_CUDA_TRY(cudaMemcpyAsync(host, dotres, 8, cudaMemcpyDeviceToHost, s));
        NGB_CUDA_TRY(cudaStreamSynchronize(s));
        *rel = std::sqrt(*host) / bn;
        return NGB_OK;
    }
    int read_scalar(const double* d, double* v, cudaStream_t s)
    {
        NGB_CUDA_TRY(cudaMemcpyAsync(host, d, 8, cudaMemcpyDeviceToHost, s));
        NGB_CUDA_TRY(cudaStreamSynchronize(s));
        *v = *host;
        return NGB_OK;
    }
};

extern "C" {

int64_t ngb_unet_weight_count(void) { return total_count(); }

int ngb_unet_write_weights(const char* path, const float* w, int64_t count)
{
    NGB_CHECK_ARG(path && w, "NULL argument");
    NGB_CHECK_ARG(count == total_count(), "weight count %lld != %lld", (long long)count, (long long)total_count());
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error("cannot open %s for writing", path);
        return NGB_ERR_INVALID;
    }
    bool           ok = std::fwrite("NGBUNET1", 1, 8, f) == 8;
    const uint32_t hdr[2] = {1u, uint32_t(kNumLayers)};
    ok = ok && std::fwrite(hdr, 4, 2, f) == 2;
    const float* p = w;
    for (int l = 0; l < kNumLayers && ok; l++) {
        const uint32_t shape[2] = {uint32_t(kLayers[l].cout), uint32_t(kLayers[l].cin)};
        ok = std::fwrite(shape, 4, 2, f) == 2;
        std::vector<uint16_t> h(size_t(layer_count(l)));
        for (size_t i = 0; i < h.size(); i++) h[i] = bf16_rne(p[i]);
        ok = ok && std::fwrite(h.data(), 2, h.size(), f) == h.size();
        p += layer_count(l);
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        set_error("write of %s failed", path);
        return NGB_ERR_INVALID;
    }
    return NGB_OK;
}

int ngb_unet_read_weights(const char* path, float* w, int64_t count)
{
    NGB_CHECK_ARG(path && w, "NULL argument");
    NGB_CHECK_ARG(count == total_count(), "weight count %lld != %lld", (long long)count, (long long)total_count());
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        set_error("cannot open %s", path);
        return NGB_ERR_INVALID;
    }
    char     magic[8];
    uint32_t hdr[2];
    bool     ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "NGBUNET1", 8) == 0 && std::fread(hdr, 4, 2, f) == 2 &&
              hdr[0] == 1u && hdr[1] == uint32_t(kNumLayers);
    float* p = w;
    for (int l = 0; l < kNumLayers && ok; l++) {
        uint32_t shape[2];
        ok = std::fread(shape, 4, 2, f) == 2 && shape[0] == uint32_t(kLayers[l].cout) && shape[1] == uint32_t(kLayers[l].cin);
        std::vector<uint16_t> h(size_t(layer_count(l)));
        ok = ok && std::fread(h.data(), 2, h.size(), f) == h.size();
        for (size_t i = 0; ok && i < h.size(); i++) p[i] = bf16_to_f32(h[i]);
        p += layer_count(l);
    }
    std::fclose(f);
    if (!ok) {
        set_error("%s is not a U-Net weight file of this library (NGBUNET1, 10 layers 16/32/64)", path);
        return NGB_ERR_INVALID;
    }
    return NGB_OK;
}

int ngb_learned_create(int32_t n, int32_t levels, const float* weights, int64_t count, ngb_learned_solver** out)
{
    NGB_CHECK_ARG(out, "NULL argument");
    *out = nullptr;
    NGB_CHECK_ARG((weights == nullptr && count == 0) || (weights && count == total_count()), "weight count %lld != %lld",
                  (long long)count, (long long)total_count());
    NGB_CHECK_ARG(levels >= 1 && levels <= 8, "levels must be in [1, 8]");
    NGB_CHECK_ARG(n > 0 && n % (1 << levels) == 0, "n must be a multiple of 2^levels");
    NGB_CHECK_ARG((n >> levels) >= 8 && (n >> levels) % 4 == 0, "the coarsest grid (n / 2^levels) must be >= 8 and a multiple of 4");
    NGB_CHECK_ARG(int64_t(n) * n * n < (int64_t(1) << 31), "n^3 must be below 2^31");
    auto* S = new ngb_learned_solver;
    auto  fail = [&](int rc) {
        delete S;
        return rc;
    };
    S->n = n;
    S->levels = levels;
    S->nc = n >> levels;
    S->net = weights != nullptr;
    const int     nc = S->nc;
    const int64_t V0 = int64_t(nc) * nc * nc, V1 = V0 / 8, V2 = V0 / 64;
    int           rc = NGB_OK;
#define NGB_ALLOC(p, bytes)                           \
    do {                                              \
        if ((rc = S->alloc(&(p), (bytes))) != NGB_OK) \
            return fail(rc);                          \
    } while (0)
    if (S->net) {
        NGB_ALLOC(S->in0, V0 * 16 * 2);
        NGB_ALLOC(S->a0, V0 * 16 * 2);
        NGB_ALLOC(S->cat0, V0 * 48 * 2);
        NGB_ALLOC(S->d0a, V0 * 16 * 2);
        NGB_ALLOC(S->out, V0 * 16 * 4);
        NGB_ALLOC(S->p0, V1 * 16 * 2);
        NGB_ALLOC(S->a1, V1 * 32 * 2);
        NGB_ALLOC(S->cat1, V1 * 96 * 2);
        NGB_ALLOC(S->d1a, V1 * 32 * 2);
        NGB_ALLOC(S->d1b, V1 * 32 * 2);
        NGB_ALLOC(S->p1, V2 * 32 * 2);
        NGB_ALLOC(S->a2, V2 * 64 * 2);
        NGB_ALLOC(S->b2, V2 * 64 * 2);
        // weights: BF16 copies (round to nearest even) and their tensor-core images
        const float* p = weights;
        for (int l = 0; l < kNumLayers; l++) {
            const size_t          cnt = size_t(layer_count(l));
            std::vector<uint16_t> h(cnt);
            for (size_t i = 0; i < cnt; i++) h[i] = bf16_rne(p[i]);
            p += cnt;
            NGB_ALLOC(S->wb[l], cnt * 2);
            NGB_ALLOC(S->wp[l], cnt * 2);
            if (cudaMemcpy(S->wb[l], h.data(), cnt * 2, cudaMemcpyHostToDevice) != cudaSuccess) {
                set_error("weight upload failed");
                return fail(NGB_ERR_CUDA);
            }
            if ((rc = ngb_conv3d_pack(kLayers[l].cout, kLayers[l].cin, S->wb[l], S->wp[l], nullptr)) != NGB_OK) return fail(rc);
        }
    }
    // V-cycle levels
    S->u.assign(levels, nullptr);
    S->tmp.assign(levels, nullptr);
    S->res.assign(levels, nullptr);
    S->r.assign(levels + 1, nullptr);
    for (int l = 0; l <= levels; l++) S->desc.push_back(box_desc(n >> l, NGB_STORE_F32, double(1 << l)));
    for (int l = 0; l < levels; l++) {
        const size_t Vl = size_t(n >> l) * (n >> l) * (n >> l);
        NGB_ALLOC(S->u[l], Vl * 4);
        NGB_ALLOC(S->tmp[l], Vl * 4);
        NGB_ALLOC(S->res[l], Vl * 4);
        const size_t Vn = size_t(n >> (l + 1)) * (n >> (l + 1)) * (n >> (l + 1));
        NGB_ALLOC(S->r[l + 1], Vn * 4);
    }
    NGB_ALLOC(S->e_c, V0 * 4);
    NGB_ALLOC(S->ae_c, V0 * 4);
    NGB_ALLOC(S->scal_c, 3 * sizeof(double));
    NGB_ALLOC(S->scratch_c, ngb_dot_scratch_doubles(V0) * sizeof(double));
    // FCG vectors
    const int64_t Vf = int64_t(n) * n * n;
    NGB_ALLOC(S->r_f, Vf * 4);
    for (int k = 0; k < 2; k++) {
        NGB_ALLOC(S->z[k], Vf * 4);
        NGB_ALLOC(S->az[k], Vf * 4);
    }
    NGB_ALLOC(S->scal, 8 * sizeof(double));
    NGB_ALLOC(S->scratch_fcg, ngb_fcg_scratch_doubles(Vf) * sizeof(double));
    NGB_ALLOC(S->scratch_dot, ngb_dot_scratch_doubles(Vf) * sizeof(double));
    NGB_ALLOC(S->dotres, sizeof(double));
    S->res_blocks = 4 * 152 * 8;
    NGB_ALLOC(S->partial, size_t(S->res_blocks) * sizeof(double));
#undef NGB_ALLOC
    if (cudaMallocHost(&S->host, 8) != cudaSuccess) {
        S->host = nullptr;
        set_error("cudaMallocHost failed");
        return fail(NGB_ERR_CUDA);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        set_error("learned solver set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(NGB_ERR_CUDA);
    }
    *out = S;
    return NGB_OK;
}

int ngb_learned_destroy(ngb_learned_solver* s)
{
    if (s) {
        cudaDeviceSynchronize();
        delete s;
    }
    return NGB_OK;
}

int ngb_learned_precondition(ngb_learned_solver* S, const float* r, float* z, void* stream)
{
    NGB_CHECK_ARG(S && r && z, "NULL argument");
    return S->cycle(0, r, z, as_stream(stream));
}

int ngb_learned_solve(ngb_learned_solver* S, const float* b, double* x, const ngb_learned_params* prm, ngb_learned_result* res,
                      void* stream)
{
    // the cycle without the network under its own range name (profiles select the learned solve by name)
    NvtxRange nvtx(S && !S->net ? "ngb_learned_solve_plain" : "ngb_learned_solve");
    NGB_CHECK_ARG(S && b && x && prm, "NULL argument");
    NGB_CHECK_ARG(prm->tol >= 0 && prm->max_iter >= 0 && prm->refresh_every >= 1 && prm->stall >= prm->refresh_every,
                  "bad params (tol >= 0, max_iter >= 0, refresh_every >= 1, stall >= refresh_every)");
    cudaStream_t  s = as_stream(stream);
    const int     n = S->n;
    const int64_t N = int64_t(n) * n * n;
    const auto    t0 = std::chrono::steady_clock::now();
    double        bb = 0.0;
    NGB_TRY(ngb_dot(N, NGB_STORE_F32, b, b, S->dotres, S->scratch_dot, s));
    NGB_TRY(S->read_scalar(S->dotres, &bb, s));
    const double bn = std::sqrt(bb);
    double       rel = 0.0;
    if (bn == 0.0) {
        NGB_CUDA_TRY(cudaMemsetAsync(x, 0, size_t(N) * 8, s));
        NGB_CUDA_TRY(cudaStreamSynchronize(s));
    } else {
        NGB_TRY(S->true_residual(b, x, bn, &rel, s));
    }
    std::vector<double> history{rel};
    const int           per = prm->stall / prm->refresh_every;
    int                 it = 0, cur = 0;
    bool                have_prev = false, fallback = false;
    while (bn > 0.0 && rel > prm->tol && it < prm->max_iter) {
        float* z = S->z[cur];
        float* az = S->az[cur];
        NGB_TRY(S->cycle(0, S->r_f, z, s));
        NGB_TRY(ngb_mg_apply(&S->desc[0], z, az, s));
        double* sc = S->scal + 2 + 2 * (it % 2);
        double* sp = S->scal + 2 + 2 * ((it + 1) % 2);
        if (have_prev) {
            NGB_TRY(ngb_dot(N, NGB_STORE_F32, z, S->az[1 - cur], S->scal, S->scratch_dot, s));
            NGB_TRY(ngb_fcg_direction(N, z, az, S->z[1 - cur], S->az[1 - cur], S->r_f, S->scal, sp, sc, S->scratch_fcg, s));
        } else {
            NGB_TRY(ngb_fcg_direction(N, z, az, nullptr, nullptr, S->r_f, nullptr, nullptr, sc, S->scratch_fcg, s));
        }
        NGB_TRY(ngb_fcg_update(N, x, z, S->r_f, az, sc, S->scal + 1, S->scratch_fcg, s));
        have_prev = true;
        cur = 1 - cur;
        it++;
        if (it % prm->refresh_every == 0) {
            NGB_TRY(ngb_conv3d_tc_check(s));
            NGB_TRY(S->true_residual(b, x, bn, &rel, s));
            history.push_back(rel);
            if (prm->fallback && int(history.size()) > per && history.back() > 0.5 * history[history.size() - 1 - per]) {
                fallback = true;
                break;
            }
        } else {
            double rr = 0.0;
            NGB_TRY(S->read_scalar(S->scal + 1, &rr, s));
            rel = std::sqrt(rr) / bn;
        }
        if (!std::isfinite(rel)) {  // breakdown (p.q zero or not finite)
            fallback = true;
            break;
        }
    }
    NGB_TRY(ngb_conv3d_tc_check(s));
    int fb_iters = 0;
    if (fallback && !(rel <= prm->tol)) {
        if (!prm->fallback) {
            set_error("learned solve broke down after %d iterations (fallback disabled)", it);
            return NGB_ERR_INVALID;
        }
        if (!std::isfinite(rel)) {
            // x may hold non-finite values: Jacobi-PCG starts from zero
            NGB_CUDA_TRY(cudaMemsetAsync(x, 0, size_t(N) * 8, s));
        }
        ngb_poisson_desc d = box_desc(n, NGB_STORE_F32, 1.0);
        const size_t     need = ngb_cg_workspace_bytes(&d);
        if (S->cg_ws_bytes < need) {
            void* w = nullptr;
            NGB_CUDA_TRY(cudaMalloc(&w, need));
            S->allocs.push_back(w);
            S->cg_ws = w;
            S->cg_ws_bytes = need;
        }
        ngb_cg_params cp{};
        cp.tol = prm->tol;
        cp.max_iter = 20000;
        cp.refresh_every = 50;
        cp.check_every = 50;
        cp.jacobi = 1;
        ngb_cg_result cr{};
        NGB_TRY(ngb_cg_solve(&d, b, x, S->cg_ws, S->cg_ws_bytes, &cp, &cr, s));
        fb_iters = cr.iterations;
        NGB_TRY(S->true_residual(b, x, bn, &rel, s));
    }
    NGB_CUDA_TRY(cudaStreamSynchronize(s));
    const auto t1 = std::chrono::steady_clock::now();
    if (res) {
        res->iterations = it;
        res->fallback = fallback ? 1 : 0;
        res->fallback_iterations = fb_iters;
        res->converged = rel <= prm->tol ? 1 : 0;
        res->rel_residual = rel;
        res->seconds = std::chrono::duration<double>(t1 - t0).count();
    }
    return NGB_OK;
}

}  // extern "C"
