// Dense LBM: FP32-compute step instantiations and the C-ABI entry points
// (step, graph-captured run, wall mask, cavity set-up, macroscopic fields).
#include "lbm_kernels.cuh"
#include <list>
#include <map>
#include <mutex>
#include <vector>
#include <cstring>

namespace ngb {

namespace {

int validate(const ngb_lbm_dense_desc* d)
{
    NGB_CHECK_ARG(d != nullptr, "desc is NULL");
    NGB_CHECK_ARG(d->q == 19 || d->q == 27, "q must be 19 or 27 (got %d)", d->q);
    NGB_CHECK_ARG(d->storage >= NGB_STORE_F64 && d->storage <= NGB_STORE_F16SR, "bad storage %d", d->storage);
    NGB_CHECK_ARG(d->nx >= 3 && d->ny >= 3 && d->nz >= 3, "dims must be >= 3 (got %d %d %d)", d->nx, d->ny, d->nz);
    NGB_CHECK_ARG(d->ny <= 65535 && d->nz <= 65535, "ny and nz must be <= 65535");
    const int64_t V = int64_t(d->nx) * d->ny * d->nz;
    NGB_CHECK_ARG(V < (int64_t(1) << 40), "lattice too large");
    NGB_CHECK_ARG(d->plane_stride == 0 || d->plane_stride >= V, "plane_stride %lld < nx*ny*nz", (long long)d->plane_stride);
    return NGB_OK;
}

inline int64_t stride_of(const ngb_lbm_dense_desc* d)
{
    return d->plane_stride ? d->plane_stride : int64_t(d->nx) * d->ny * d->nz;
}

template <typename C, typename S>
C round_through(double v)
{
    return C(S(v));
}

DenseParams<float> params_f32(const ngb_lbm_dense_desc* d, uint32_t step = 0)
{
    DenseParams<float> p{};
    p.seed = d->dither_seed + step;
    p.nx = d->nx, p.ny = d->ny, p.nz = d->nz, p.box = d->box_cavity ? 1 : 0, p.stride = stride_of(d);
    p.omega = float(d->omega);
    for (int c = 0; c < 2; c++)
        for (int q = 0; q < 27; q++) p.wall[c][q] = float(d->wall_term[c][q]);
    p.zh_rho = float(d->zouhe_rho - 1.0);  // the shifted form works on rho - 1
    for (int a = 0; a < 3; a++) p.zh_u[a] = float(d->zouhe_u[a]);
    return p;
}

DenseParams<double> params_f64(const ngb_lbm_dense_desc* d)
{
    DenseParams<double> p{};
    p.nx = d->nx, p.ny = d->ny, p.nz = d->nz, p.box = d->box_cavity ? 1 : 0, p.stride = stride_of(d);
    p.omega = d->omega;
    for (int c = 0; c < 2; c++)
        for (int q = 0; q < 27; q++) p.wall[c][q] = d->wall_term[c][q];
    p.zh_rho = d->zouhe_rho;
    for (int a = 0; a < 3; a++) p.zh_u[a] = d->zouhe_u[a];
    return p;
}

// `step`: index of the step within a run (its dither seed is dither_seed + step).
int step_impl(const ngb_lbm_dense_desc* d, const void* fin, void* fout, const uint32_t* flags, cudaStream_t s, uint32_t step = 0)
{
    if (d->storage == NGB_STORE_F64) return launch_lbm_dense_f64(d->q, fin, fout, flags, params_f64(d), s);
    return launch_lbm_dense_f32(d->q, d->storage, fin, fout, flags, params_f32(d, step), s);
}

// ---------------------------------------------------------------- graph cache for ngb_lbm_dense_run
struct RunKey {
    ngb_lbm_dense_desc desc;
    const void*        fa;
    const void*        fb;
    const uint32_t*    flags;
    int                steps;
    bool operator<(const RunKey& o) const { return std::memcmp(this, &o, sizeof(RunKey)) < 0; }
};
// Least-recently-used cache of instantiated step graphs, bounded so that
// callers that reallocate their population buffers do not accumulate graphs.
// An evicted graph may still be running on a stream: cudaGraphExecDestroy
// then frees it once that launch completes.
struct RunCache {
    std::list<std::pair<RunKey, cudaGraphExec_t>>                                    lru;  // front = newest
    std::map<RunKey, std::list<std::pair<RunKey, cudaGraphExec_t>>::iterator>        index;
};
std::mutex    g_run_mutex;
RunCache      g_run_graphs;
constexpr int kStepsPerGraph = 32;  // even: the graph ends on the buffer it started from
constexpr int kMaxRunGraphs = 8;

void release_run_graphs_locked()
{
    for (auto& e : g_run_graphs.lru) cudaGraphExecDestroy(e.second);
    g_run_graphs.lru.clear();
    g_run_graphs.index.clear();
}

int get_run_graph(const RunKey& k, cudaGraphExec_t& exec)
{
    auto it = g_run_graphs.index.find(k);
    if (it != g_run_graphs.index.end()) {
        g_run_graphs.lru.splice(g_run_graphs.lru.begin(), g_run_graphs.lru, it->second);
        exec = it->second->second;
        return NGB_OK;
    }
    cudaStream_t cs;
    NGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int         rc = NGB_OK;
    if (e == cudaSuccess) {
        for (int t = 0; t < k.steps && rc == NGB_OK; t++)
            rc = step_impl(&k.desc, t % 2 == 0 ? k.fa : k.fb, const_cast<void*>(t % 2 == 0 ? k.fb : k.fa), k.flags, cs,
                           uint32_t(t));
        e = cudaStreamEndCapture(cs, &graph);
    }
    cudaStreamDestroy(cs);
    if (rc != NGB_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) {
        set_error("graph capture failed: %s", cudaGetErrorString(e));
        return NGB_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error("graph instantiate failed: %s", cudaGetErrorString(e));
        return NGB_ERR_CUDA;
    }
    g_run_graphs.lru.emplace_front(k, exec);
    g_run_graphs.index[k] = g_run_graphs.lru.begin();
    while (int(g_run_graphs.lru.size()) > kMaxRunGraphs) {
        cudaGraphExecDestroy(g_run_graphs.lru.back().second);
        g_run_graphs.index.erase(g_run_graphs.lru.back().first);
        g_run_graphs.lru.pop_back();
    }
    return NGB_OK;
}

// ---------------------------------------------------------------- set-up kernels
template <int Q>
__global__ void wall_mask_kernel(uint32_t* flags, int nx, int ny, int nz)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= nx) return;
    const int64_t  sy = nx, sz = int64_t(nx) * ny, cell = x + sy * y + sz * z;
    const uint32_t f = flags[cell];
    const int      cls = flag_class(f);
    if (cls != NGB_CELL_BULK && !is_zouhe_class(cls)) {  // Zou-He nodes are updated and need the mask too
        flags[cell] = make_flag(0, cls);
        return;
    }
    uint32_t mask = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int cx = Lattice<Q>::cx(q), cy = Lattice<Q>::cy(q), cz = Lattice<Q>::cz(q);
        if (cx == 0 && cy == 0 && cz == 0) continue;
        const int sx = x - cx, syy = y - cy, szz = z - cz;
        bool      wall = true;  // outside the domain counts as "undefined"
        if (sx >= 0 && syy >= 0 && szz >= 0 && sx < nx && syy < ny && szz < nz)
            wall = !is_fluid_class(flag_class(flags[sx + sy * syy + sz * szz]));
        if (wall) mask |= 1u << q;
    }
    flags[cell] = make_flag(mask, cls);
}

template <int Q, typename S>
__global__ void cavity_init_kernel(S* fa, S* fb, uint32_t* flags, int nx, int ny, int nz, int64_t stride, double ulb, int off)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= nx) return;
    const int64_t cell = x + int64_t(nx) * (y + int64_t(ny) * z);
    const bool    face = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
    const bool    lid = y == ny - 1;
    if (flags) flags[cell] = make_flag(0, face ? (lid ? NGB_CELL_MOVINGWALL : NGB_CELL_BOUNCEBACK) : NGB_CELL_BULK);
#pragma unroll
    for (int q = 0; q < Q; q++) {
        double v = Lattice<Q>::w(q);
        if (face) v = lid ? -6. * Lattice<Q>::w(q) * ulb * double(Lattice<Q>::cx(q)) : 0.0;
        S sv;
        if (off) {
            sv = S(0.0f);  // g = f - w = 0 on fluid nodes; wall nodes use the wall table
        } else {
            sv = S(v);
        }
        if (fa) fa[q * stride + cell] = sv;
        if (fb) fb[q * stride + cell] = sv;
    }
}

template <typename S>
__device__ __forceinline__ double pop_value(const S* p, double w, int off)
{
    if constexpr (std::is_same<S, double>::value || std::is_same<S, float>::value) {
        return double(*p);
    } else if constexpr (std::is_same<S, __half>::value) {
        return double(__half2float(*p) * (1.0f / NGB_F16OFF_SCALE)) + double(float(w));
    } else {
        return double(__bfloat162float(*p)) + double(float(w));
    }
}

template <int Q, typename S>
__global__ void macroscopic_kernel(const S* __restrict__ fin, const uint32_t* __restrict__ flags, DenseParams<double> p,
                                   double* rho_out, double* u_out)
{
    using L = Lattice<Q>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= p.nx) return;
    const int64_t sy = p.nx, sz = int64_t(p.nx) * p.ny, V = sz * p.nz, cell = x + sy * y + sz * z;
    uint32_t      mask, lidbits;
    const int     cls = cell_setup<Q>(p, flags, x, y, z, cell, mask, lidbits);
    double        rho = 0, u[3] = {0, 0, 0};
    if (cls == NGB_CELL_BULK) {
        double m[3] = {0, 0, 0};
        for (int q = 0; q < Q; q++) {
            double f;
            if (mask & (1u << q)) {
                const int o = L::opp(q);
                f = pop_value(fin + o * p.stride + cell, L::w(o), 0) + ((lidbits >> q) & 1u ? p.wall[1][o] : p.wall[0][o]);
            } else {
                const int64_t src = cell - L::cx(q) - L::cy(q) * sy - L::cz(q) * sz;
                f = pop_value(fin + q * p.stride + src, L::w(q), 0);
            }
            rho += f;
            m[0] += L::cx(q) * f, m[1] += L::cy(q) * f, m[2] += L::cz(q) * f;
        }
        for (int a = 0; a < 3; a++) u[a] = m[a] / rho;
    } else if (cls == NGB_CELL_MOVINGWALL) {
        // LbmTools.h:411-427: rho = 1, u_a = f_a / (6 * 1/18) for a = 0, 1, 2 (D3Q19 order)
        rho = 1.0;
        for (int a = 0; a < 3; a++) u[a] = p.wall[1][Q == 19 ? a : 0] / (6. * 1. / 18.);
        if (Q != 19) u[0] = u[1] = u[2] = 0;
    }
    if (rho_out) rho_out[cell] = rho;
    if (u_out)
        for (int a = 0; a < 3; a++) u_out[a * V + cell] = u[a];
}

}  // namespace
}  // namespace ngb

using namespace ngb;

extern "C" {

int ngb_lbm_dense_step(const ngb_lbm_dense_desc* d, const void* fin, void* fout, const uint32_t* flags, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(fin && fout && fin != fout, "fin/fout must be distinct non-NULL device pointers");
    NGB_CHECK_ARG(d->box_cavity || flags, "flags required when box_cavity == 0");
    return step_impl(d, fin, fout, flags, as_stream(stream));
}

int ngb_lbm_dense_kernels_per_step(const ngb_lbm_dense_desc* d)
{
    int rc = validate(d);
    if (rc) return rc;
    if (d->storage == NGB_STORE_F64) return 1;
    return lbm_dense_split(d->q, d->storage, params_f32(d)) ? 2 : 1;
}

int ngb_lbm_dense_run(const ngb_lbm_dense_desc* d, void* fa, void* fb, const uint32_t* flags, int32_t nsteps, void* stream)
{
    NvtxRange nvtx("ngb_lbm_dense_run");
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(fa && fb && fa != fb, "fa/fb must be distinct non-NULL device pointers");
    NGB_CHECK_ARG(d->box_cavity || flags, "flags required when box_cavity == 0");
    NGB_CHECK_ARG(nsteps >= 0, "nsteps < 0");
    cudaStream_t s = as_stream(stream);
    const int    full = nsteps / kStepsPerGraph;
    const int    rest = nsteps % kStepsPerGraph;
    RunKey       k;
    std::memset(&k, 0, sizeof(k));
    k.desc = *d, k.fa = fa, k.fb = fb, k.flags = d->box_cavity ? nullptr : flags;
    if (full > 0) {
        std::lock_guard<std::mutex> lock(g_run_mutex);
        k.steps = kStepsPerGraph;
        cudaGraphExec_t exec;
        rc = get_run_graph(k, exec);
        if (rc) return rc;
        for (int i = 0; i < full; i++) NGB_CUDA_TRY(cudaGraphLaunch(exec, s));
    }
    for (int t = 0; t < rest; t++) {  // steps 32 full + t: seed offset t (mod 32)
        rc = step_impl(d, t % 2 == 0 ? fa : fb, t % 2 == 0 ? fb : fa, flags, s, uint32_t(t));
        if (rc) return rc;
    }
    return NGB_OK;
}

int ngb_lbm_dense_run_host(const ngb_lbm_dense_desc* d, const void* host_in, void* host_out, void* fa, void* fb,
                           const uint32_t* flags, int32_t nsteps, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(host_in && host_out, "host buffers must be non-NULL");
    const size_t bytes = size_t(d->q) * size_t(stride_of(d)) * storage_bytes(d->storage);
    cudaStream_t s = as_stream(stream);
    NGB_CUDA_TRY(cudaMemcpyAsync(fa, host_in, bytes, cudaMemcpyHostToDevice, s));
    // After an odd count the result is fb, whose non-bulk nodes no step
    // writes: give fb the uploaded state first (both ping-pong buffers start
    // identical, as RunCavityTwoPop.cu:168-206 initialises them).
    if (nsteps % 2 == 1) NGB_CUDA_TRY(cudaMemcpyAsync(fb, fa, bytes, cudaMemcpyDeviceToDevice, s));
    rc = ngb_lbm_dense_run(d, fa, fb, flags, nsteps, stream);
    if (rc) return rc;
    NGB_CUDA_TRY(cudaMemcpyAsync(host_out, nsteps % 2 == 0 ? fa : fb, bytes, cudaMemcpyDeviceToHost, s));
    return NGB_OK;
}

int ngb_lbm_release_graphs(void)
{
    std::lock_guard<std::mutex> lock(g_run_mutex);
    release_run_graphs_locked();
    return NGB_OK;
}

int ngb_lbm_wall_mask(int32_t nx, int32_t ny, int32_t nz, int32_t q, uint32_t* flags, void* stream)
{
    NGB_CHECK_ARG(q == 19 || q == 27, "q must be 19 or 27");
    NGB_CHECK_ARG(nx > 0 && ny > 0 && nz > 0 && ny <= 65535 && nz <= 65535 && flags, "bad dims or NULL flags");
    const dim3 grid((nx + 127) / 128, ny, nz), block(128);
    if (q == 19)
        wall_mask_kernel<19><<<grid, block, 0, as_stream(stream)>>>(flags, nx, ny, nz);
    else
        wall_mask_kernel<27><<<grid, block, 0, as_stream(stream)>>>(flags, nx, ny, nz);
    NGB_LAUNCH_CHECK("wall_mask_kernel");
    return NGB_OK;
}

int ngb_lbm_cavity_init(const ngb_lbm_dense_desc* d, double ulb, void* fa, void* fb, uint32_t* flags, void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    const dim3   grid((d->nx + 127) / 128, d->ny, d->nz), block(128);
    const int64_t st = stride_of(d);
#define NGB_INIT(QQ, T, OFF)                                                                                                   \
    cavity_init_kernel<QQ, T><<<grid, block, 0, s>>>(static_cast<T*>(fa), static_cast<T*>(fb), flags, d->nx, d->ny, d->nz, st, \
                                                     ulb, OFF)
    const bool q19 = d->q == 19;
    switch (d->storage) {
        case NGB_STORE_F64:
            if (q19) NGB_INIT(19, double, 0); else NGB_INIT(27, double, 0);
            break;
        case NGB_STORE_F32:
            if (q19) NGB_INIT(19, float, 0); else NGB_INIT(27, float, 0);
            break;
        case NGB_STORE_F16OFF:
        case NGB_STORE_F16SR:
            if (q19) NGB_INIT(19, __half, 1); else NGB_INIT(27, __half, 1);
            break;
        default:
            if (q19) NGB_INIT(19, __nv_bfloat16, 1); else NGB_INIT(27, __nv_bfloat16, 1);
            break;
    }
#undef NGB_INIT
    NGB_LAUNCH_CHECK("cavity_init_kernel");
    if (flags) return ngb_lbm_wall_mask(d->nx, d->ny, d->nz, d->q, flags, stream);
    return NGB_OK;
}

int ngb_lbm_dense_macroscopic(const ngb_lbm_dense_desc* d, const void* fin, const uint32_t* flags, double* rho, double* u,
                              void* stream)
{
    int rc = validate(d);
    if (rc) return rc;
    NGB_CHECK_ARG(fin, "fin is NULL");
    NGB_CHECK_ARG(d->box_cavity || flags, "flags required when box_cavity == 0");
    DenseParams<double> p = params_f64(d);
    // wall terms as the step sees them: rounded through the storage type
    for (int c = 0; c < 2; c++)
        for (int q = 0; q < 27; q++)
            p.wall[c][q] = d->storage == NGB_STORE_F64 ? d->wall_term[c][q] : double(float(d->wall_term[c][q]));
    cudaStream_t s = as_stream(stream);
    const dim3   grid((d->nx + 127) / 128, d->ny, d->nz), block(128);
#define NGB_MAC(QQ, T) macroscopic_kernel<QQ, T><<<grid, block, 0, s>>>(static_cast<const T*>(fin), flags, p, rho, u)
    const bool q19 = d->q == 19;
    switch (d->storage) {
        case NGB_STORE_F64:
            if (q19) NGB_MAC(19, double); else NGB_MAC(27, double);
            break;
        case NGB_STORE_F32:
            if (q19) NGB_MAC(19, float); else NGB_MAC(27, float);
            break;
        case NGB_STORE_F16OFF:
        case NGB_STORE_F16SR:
            if (q19) NGB_MAC(19, __half); else NGB_MAC(27, __half);
            break;
        default:
            if (q19) NGB_MAC(19, __nv_bfloat16); else NGB_MAC(27, __nv_bfloat16);
            break;
    }
#undef NGB_MAC
    NGB_LAUNCH_CHECK("macroscopic_kernel");
    return NGB_OK;
}

}  // extern "C"
