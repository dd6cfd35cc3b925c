/*
 * neon_gb300 — C ABI of the GB300-native Neon grid-stencil path.
 *
 * Plain pointers and sizes only. Every function returns an ngb status
 * (NGB_OK = 0, negative on error) and never throws; the message of the last
 * error of the calling host thread is returned by ngb_last_error().
 * Device pointers are CUDA global-memory pointers on the current device;
 * `stream` is a cudaStream_t (NULL = legacy default stream). All calls that
 * take a stream are asynchronous with respect to the host unless stated.
 *
 * Each entry point names the Neon interface it replaces (paths relative to
 * the Neon repository).
 */
#ifndef NEON_GB300_H
#define NEON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NGB_OK 0
#define NGB_ERR_INVALID (-1)     /* bad argument (size, pointer, enum) */
#define NGB_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define NGB_ERR_UNSUPPORTED (-3) /* valid but not implemented combination */
#define NGB_ERR_RANGE (-4)       /* size beyond a stated maximum */
#define NGB_ERR_TIMEOUT (-5)     /* a bounded device-side wait gave up */

/* Message of the last failed call on this host thread ("" if none). */
const char* ngb_last_error(void);
/* ABI version of the loaded library. */
int ngb_version(void);
/* sizeof of the ABI structs, for bindings that lay them out themselves:
 * 0 ngb_lbm_dense_desc, 1 ngb_bgrid_desc, 2 ngb_poisson_desc, 3 ngb_cg_params,
 * 4 ngb_cg_result, 5 ngb_learned_params, 6 ngb_learned_result; 0 otherwise. */
size_t ngb_abi_struct_size(int32_t which);

/* ------------------------------------------------------------------------
 * Lattice-Boltzmann populations
 * ---------------------------------------------------------------------- */

/* How populations are held in HBM. The *_OFF forms hold g_q = f_q - w_q:
 * BF16OFF as bf16(g_q); F16OFF as fp16(2^14 g_q) (NGB_F16OFF_SCALE), which
 * keeps the small offsets of slow flow regions out of FP16's subnormal range
 * (2^14 is exact, so the FP32 collision computes the same values either way).
 * F16SR holds the same fp16(2^14 g_q) values but stores them with stochastic
 * rounding: the FP32 result is rounded up in magnitude with probability
 * equal to its remainder, so the rounding errors of a quasi-steady flow do
 * not add up to a systematic drift (round-to-nearest repeats the same error
 * every step). The random bits are a hash of the cell, the population and
 * the step seed: for cell index i (x + nx (y + ny z)), population q and seed s,
 *   h  = mix32(lo32(i >> 1) ^ (hi32(i >> 1) * 0x9E3779B1) ^ (s * 0x85EBCA77)),
 *   hq = (h ^ (q * 0x9E3779B9)) * 0xC2B2AE35,
 *   r  = i odd ? (hq >> 16) & 0x1FFF : hq & 0x1FFF    (13 bits)
 * with mix32(x) = x ^= x >> 16, x *= 0x7FEB352D, x ^= x >> 15,
 * x *= 0x846CA68B, x ^= x >> 16 (Wellons' "lowbias32"); the stored value is
 * 2^14 g with r / 2^13 of its FP16 ulp added to the magnitude, then
 * truncated (FP16 subnormals included): the GPU's cvt.rs.f16x2.f32 with hq as
 * the random word of the pair (2i, 2i+1). ngb_lbm_dense_step uses
 * s = dither_seed; the t-th step of ngb_lbm_dense_run uses
 * s = dither_seed + (t mod 32). */
#define NGB_F16OFF_SCALE 16384.0f
typedef enum {
    NGB_STORE_F64 = 0,
    NGB_STORE_F32 = 1,
    NGB_STORE_F16OFF = 2,
    NGB_STORE_BF16OFF = 3,
    NGB_STORE_F16SR = 4
} ngb_storage;

/* Cell classification, values of benchmarks/lbm-lid-driven-cavity-flow/src/CellType.h:5-11
 * plus OUTLET (zero-gradient outflow node, new) and the Zou-He pressure /
 * velocity boundary nodes of benchmarks/lbm-flow-over-sphere/src/CellType.h
 * (PRESSURE, VELOCITY; D3Q19 on dense grids with a flag array, FP64 and FP32
 * storage). A Zou-He node lies on a face of the box and is updated every step:
 * with n its inward normal (the first face it lies on, in the order x = 0,
 * x = nx-1, y = 0, y = ny-1, z = 0, z = nz-1), the 5 populations with
 * c.n = +1 are unknown; M and K are the sums of the known populations with
 * c.n = 0 and c.n = -1; PRESSURE nodes take rho = zouhe_rho, u.n =
 * 1 - (M + 2K) / rho and zero tangential velocity, VELOCITY nodes take u =
 * zouhe_u and rho = (M + 2K) / (1 - u.n); the unknowns are
 * f_q = f_opp(q) + eq_q - eq_opp(q) (non-equilibrium bounce-back, Zou & He
 * 1997) and the node collides with eq(rho, u) of those boundary values. */
typedef enum {
    NGB_CELL_BOUNCEBACK = 0,
    NGB_CELL_MOVINGWALL = 1,
    NGB_CELL_BULK = 2,
    NGB_CELL_UNDEFINED = 3,
    NGB_CELL_OUTLET = 4,
    NGB_CELL_PRESSURE = 5,
    NGB_CELL_VELOCITY = 6
} ngb_cell_class;

/* Packed cell flag (uint32 per cell): bits 0..26 = wall-neighbour mask
 * (bit q set iff the pull source x - c_q is not a fluid node),
 * bits 28..31 = ngb_cell_class. Replaces the 8-byte CellType
 * {wallNghBitflag, classification} of CellType.h:3-35. */
#define NGB_FLAG_MASK(f) ((f) & 0x07ffffffu)
#define NGB_FLAG_CLASS(f) ((int)((f) >> 28))
#define NGB_MAKE_FLAG(mask, cls) (((mask) & 0x07ffffffu) | ((uint32_t)(cls) << 28))

/* Dense single-partition lattice. Population (x, y, z, q) lives at element
 * x + nx*(y + ny*z) + q*plane_stride, the SoA layout of a single-partition
 * Neon dField (libNeonDomain/include/Neon/domain/details/dGrid/dField_imp.h:71-87). */
typedef struct ngb_lbm_dense_desc {
    int32_t nx, ny, nz;
    int32_t q;            /* 19 (D3Q19, Neon order of D3Q19.h:23-44) or 27 (order of apps/lbmMultiRes/lattice.h:14-42) */
    int32_t storage;      /* ngb_storage */
    int32_t box_cavity;   /* 1: classification and wall mask follow from coordinates (box faces are
                             bounce-back walls, y = ny-1 the moving lid, RunCavityTwoPop.cu:208-224);
                             0: read from the packed flag array */
    int64_t plane_stride; /* elements between population planes; 0 means nx*ny*nz */
    double  omega;        /* BGK relaxation rate */
    /* Population held by a wall node, by the wall's classification:
     * [0] bounce-back, [1] moving wall (RunCavityTwoPop.cu:168-186 stores
     * -6 w_k u_lb (c_k . u_lid) on the lid, 0 elsewhere). Rounded to the
     * storage precision (F64/F32) or kept in FP32 (*_OFF) by the library. */
    double wall_term[2][27];
    double   zouhe_rho;   /* density of the PRESSURE nodes */
    double   zouhe_u[3];  /* velocity of the VELOCITY nodes */
    uint32_t dither_seed; /* F16SR: seed of the stochastic rounding (see ngb_storage) */
    uint32_t pad;
} ngb_lbm_dense_desc;

/* One pull stream-collide step over every bulk cell: fout <- step(fin).
 * Non-bulk cells of fout are left untouched; outlet cells copy the
 * populations of their x-1 neighbour.
 * Replaces LbmContainers<D3Q19>::iteration (benchmarks/lbm-lid-driven-cavity-flow/src/LbmTools.h:284-325)
 * run through Skeleton::run (libNeonSkeleton/include/Neon/skeleton/Skeleton.h:56-65).
 * F64 storage computes with the reference's arithmetic in FP64; the other
 * storages compute in FP32 on equilibrium-shifted values. */
int ngb_lbm_dense_step(const ngb_lbm_dense_desc* desc, const void* fin, void* fout, const uint32_t* flags, void* stream);

/* `nsteps` steps ping-ponging fa -> fb -> fa ...; after an odd count the
 * newest populations are in fb. Launches are captured once into a CUDA graph
 * per (desc, pointers) and replayed; the library keeps the 8 most recently
 * used graphs and destroys older ones. Replaces the host loop of
 * RunCavityTwoPop.cu:257-273 over LbmIterationD3Q19::run (LbmIteration.h:56-61). */
int ngb_lbm_dense_run(const ngb_lbm_dense_desc* desc, void* fa, void* fb, const uint32_t* flags, int32_t nsteps, void* stream);

/* Checkpoint / resume (no reference counterpart; the reference exports
 * VTK/VTI only, FieldBase.h:137). save writes the population buffer f (the
 * newest state, q * plane_stride elements) after a header with the lattice
 * dims, q, storage, plane stride, omega and the caller's step number
 * ("NGBLBM01", little-endian). load checks the header against desc, fills fa
 * and, when fb is non-NULL, fb with the saved state (both ping-pong buffers
 * equal, as a fresh run starts, so the continued run is bit-identical) and
 * returns the step number. Both are synchronous (file IO through a pinned
 * 64 MiB staging buffer). */
int ngb_lbm_dense_save(const char* path, const ngb_lbm_dense_desc* desc, const void* f, int64_t step, void* stream);
int ngb_lbm_dense_load(const char* path, const ngb_lbm_dense_desc* desc, void* fa, void* fb, int64_t* step, void* stream);

/* Destroys every step graph ngb_lbm_dense_run keeps (a graph still running
 * is freed when its launch completes). Call before freeing population
 * buffers for good, or to return the graphs' memory. No reference
 * counterpart (the reference launches without graphs). */
int ngb_lbm_release_graphs(void);

/* Kernel launches one step of `desc` issues (1, or 2 where the analytic
 * cavity runs as a core + wall-shell kernel pair): launch accounting for
 * callers that size graphs or count kernels. No reference counterpart.
 * Returns a negative status for an invalid desc. */
int ngb_lbm_dense_kernels_per_step(const ngb_lbm_dense_desc* desc);

/* Host-buffer form of ngb_lbm_dense_run for callers whose populations live
 * in host memory: copies host_in (pinned or pageable, q*plane_stride
 * elements) into fa (and, for an odd nsteps, on into fb, whose non-bulk
 * nodes the steps never write), runs nsteps, and copies the newest
 * populations back to host_out; fa/fb are caller-provided device buffers. Stream-ordered; the
 * host buffers must stay valid until the stream reaches this point.
 * Replaces Field::updateDeviceData / run loop / Field::updateHostData
 * (dField_imp.h, RunCavityTwoPop.cu:226-273). */
int ngb_lbm_dense_run_host(const ngb_lbm_dense_desc* desc, const void* host_in, void* host_out, void* fa, void* fb,
                           const uint32_t* flags, int32_t nsteps, void* stream);

/* Wall-neighbour mask from the classifications in `flags` (in place):
 * replaces LbmContainers::computeWallNghMask (LbmTools.h:327-376). */
int ngb_lbm_wall_mask(int32_t nx, int32_t ny, int32_t nz, int32_t q, uint32_t* flags, void* stream);

/* Cavity set-up on the device (RunCavityTwoPop.cu:159-242): populations
 * of both buffers (either may be NULL) and, if non-NULL, the packed flags
 * with their wall mask. `ulb` is the lid speed along +x. */
int ngb_lbm_cavity_init(const ngb_lbm_dense_desc* desc, double ulb, void* fa, void* fb, uint32_t* flags, void* stream);

/* Density and velocity of every bulk cell (rho: V values, u: 3 planes of V),
 * in double, computed by pulling populations like the step does; moving-wall
 * cells get rho = 1 and u from their stored lid term; other cells 0.
 * Replaces LbmContainers::computeRhoAndU (LbmTools.h:383-437). */
int ngb_lbm_dense_macroscopic(const ngb_lbm_dense_desc* desc, const void* fin, const uint32_t* flags, double* rho,
                              double* u, void* stream);

/* ------------------------------------------------------------------------
 * Block-sparse grid (bGrid, 8x8x8 blocks), single partition
 * ---------------------------------------------------------------------- */

/* ------------------------------------------------------------------------
 * Element-sparse grid (eGrid), single partition
 * ---------------------------------------------------------------------- */

/* int32 scratch entries ngb_egrid_count needs. */
#define NGB_EGRID_SCRATCH(nx, ny, nz) ((((int64_t)(nx) * (ny) * (nz)) + 2047) / 2048 + 1)

/* Phase 1 of the eGrid construction on the device (eGrid_imp.h:8-129, which
 * runs Partitioner1D at block size 1; one partition: every active cell is an
 * internal element, in the order z, then y, then x fastest,
 * SpanClassifier.h:228-237). `active` is a dense nx*ny*nz byte map (x
 * fastest, non-zero = active). elem_of[nx*ny*nz] receives each cell's element
 * index or -1, *count (device) the number of elements; `scratch` holds
 * NGB_EGRID_SCRATCH(nx, ny, nz) int32. Fewer than 2^31 cells. */
int ngb_egrid_count(int32_t nx, int32_t ny, int32_t nz, const uint8_t* active, int32_t* elem_of, int32_t* scratch, int32_t* count,
                    void* stream);

/* Phase 2: origin[3*count] = (x, y, z) of every element (the global mapping of
 * Partitioner1D.h:212-255) and, for the `npts` stencil offsets in `points`
 * (host, 3 int8 per point, in the stencil's neighbour order, at most 64),
 * conn[s*count + e] = the element at origin[e] + points[s], or -1 outside the
 * grid or on an inactive cell (Partitioner1D.h:338-380; read by
 * ePartition_imp.h isValidNgh). */
int ngb_egrid_fill(int32_t nx, int32_t ny, int32_t nz, const int32_t* elem_of, int32_t count, const int8_t* points, int32_t npts,
                   int32_t* origin, int32_t* conn, void* stream);

/* Candidate blocks per axis: ceil(n / 8). */
#define NGB_BGRID_BLOCKS(n) (((n) + 7) / 8)
#define NGB_BGRID_NO_BLOCK 0xffffffffu

/* Phase 1 of the bGrid construction on the device. `active` is a dense
 * nx*ny*nz byte map (x fastest, non-zero = active voxel). Fills
 * block_of[bnx*bny*bnz] (x fastest) with the data-block index of every
 * candidate block, or -1 when none of its voxels is inside the domain and
 * active, and writes the number of data blocks to *n_blocks (device) .
 * Data-block order is the single-partition order of Neon: z, then y, then x
 * fastest over candidate blocks (SpanDecomposition.h:71-96,
 * SpanClassifier.h:228-237, SpanClassifier.cpp:7-20). */
int ngb_bgrid_count(int32_t nx, int32_t ny, int32_t nz, const uint8_t* active, int32_t* block_of, uint32_t* n_blocks,
                    void* stream);

/* Phase 2: per data block, origin (3 x int32: block index * 8,
 * Partitioner1D.h:212-255), active bitmask (16 x uint32, bit x + 8y + 64z,
 * bGrid_imp.h:80-136 / StaticBlock.h:79-98) and 27-entry connectivity
 * (entry i + 3j + 9k = data block at offset (i-1, j-1, k-1) or
 * NGB_BGRID_NO_BLOCK, bGrid_imp.h:139-172). n_active_voxels (device,
 * uint64) receives the active-voxel count. Arrays hold n_blocks entries. */
int ngb_bgrid_fill(int32_t nx, int32_t ny, int32_t nz, const uint8_t* active, const int32_t* block_of, int32_t* origin,
                   uint32_t* mask, uint32_t* conn, unsigned long long* n_active_voxels, void* stream);

/* Block-sparse lattice. Population (block b, voxel i + 8j + 64k, q) lives
 * at ((b*q + q)*512 + i + 8j + 64k) — per-block SoA as a Neon bField
 * (bPartition_imp.h:95-107). A neighbour that is outside every data block or
 * not active counts as a non-fluid node ("undefined"), as bPartition's
 * invalid NghData does (bPartition_imp.h:109-124). */
typedef struct ngb_bgrid_desc {
    int32_t         n_blocks;
    int32_t         q;       /* 19 or 27 */
    int32_t         storage; /* ngb_storage */
    int32_t         pad;
    double          omega;
    double          wall_term[2][27]; /* as ngb_lbm_dense_desc */
    const int32_t*  origin;           /* device arrays from ngb_bgrid_fill */
    const uint32_t* mask;
    const uint32_t* conn;
} ngb_bgrid_desc;

/* Wall-neighbour mask of every bulk voxel of a bGrid flag field (uint32 per
 * voxel, per-block layout b*512 + i + 8j + 64k), in place; classifications
 * are kept. Same rule as ngb_lbm_wall_mask with bGrid neighbour resolution. */
int ngb_bgrid_wall_mask(const ngb_bgrid_desc* desc, uint32_t* flags, void* stream);

/* One pull stream-collide step on a bGrid: replaces LbmContainers::iteration
 * on Neon::bGrid (LbmTools.h:284-325 run through blockSpan::launchLambdaOnSpanCUDA,
 * LambdaExecutor.h:103-115). Same arithmetic as ngb_lbm_dense_step. */
int ngb_bgrid_lbm_step(const ngb_bgrid_desc* desc, const void* fin, void* fout, const uint32_t* flags, void* stream);

/* Momentum-exchange force (3 doubles, device) on every bounce-back node, from
 * the populations `fin` that the next step reads: F = sum over bulk voxels x
 * and directions q whose pull source x - c_q is a bounce-back node of
 * 2 c_{opp q} f_{opp q}(x). New (the reference computes no drag).
 * Deterministic: fixed per-block partials reduced in block order; `partials`
 * is caller scratch of 3 * n_blocks doubles. */
int ngb_bgrid_drag(const ngb_bgrid_desc* desc, const void* fin, const uint32_t* flags, double* partials, double* force,
                   void* stream);

/* Geometry of the flow-over-sphere case on a dense byte map: voxel active
 * iff within `band` of the sphere surface (or inside it) or within
 * `tube_band` of a tube of radius `tube_r` whose axis runs along x through
 * control points every `ctrl_dx` voxels at (y, z) = tube_c + amplitude *
 * (2u - 1), u from std::mt19937_64(seed) (53-bit uniforms, y then z per
 * point), linearly interpolated. Classes (uint8 per voxel): bounce-back
 * inside the sphere, moving wall (inlet) at x = 0, outlet at x = nx-1, bulk
 * otherwise; inactive voxels get NGB_CELL_UNDEFINED. */
typedef struct ngb_sphere_tube {
    int32_t  nx, ny, nz;
    int32_t  ctrl_dx;
    double   sphere_c[3];
    double   sphere_r;
    double   band;
    double   tube_c[2];
    double   tube_r;
    double   tube_band;
    double   amplitude;
    uint64_t seed;
} ngb_sphere_tube;
int ngb_geometry_sphere_tube(const ngb_sphere_tube* g, uint8_t* active, uint8_t* cls, void* stream);

/* Scatter a dense per-voxel uint8 class map into a bGrid flag field
 * (classification only, mask 0): flags[b*512 + v] = class of the voxel. */
int ngb_bgrid_flags_from_dense(const ngb_bgrid_desc* desc, int32_t nx, int32_t ny, int32_t nz, const uint8_t* cls,
                               uint32_t* flags, void* stream);

/* Integer 6-neighbour operator of Neon's domain-stencil tests on a bGrid
 * (TestData::laplace, TestData.h:412-443, through bPartition::getNghData):
 * b = a - count * sum of valid neighbours, int64, cardinality 1. */
int ngb_bgrid_laplace_i64(const ngb_bgrid_desc* desc, const int64_t* a, int64_t* b, void* stream);

/* Same operator on a dense single-partition dGrid (validity = inside the box,
 * dPartition.h:228-263). */
int ngb_dense_laplace_i64(int32_t nx, int32_t ny, int32_t nz, const int64_t* a, int64_t* b, void* stream);

/* ------------------------------------------------------------------------
 * Poisson: 7-point Laplacian and (Jacobi-preconditioned) CG
 * ---------------------------------------------------------------------- */

/* Dense single-partition scalar field (x fastest). `field` is NGB_STORE_F32
 * or NGB_STORE_F64. `bd` marks each cell Fixed (0, Dirichlet) or Free (1)
 * as libNeonSolver's BoundaryCondition (IterativeLinearSolver.h:17-21);
 * NULL means every box-face cell is Fixed and every other cell Free. */
typedef struct ngb_poisson_desc {
    int32_t       nx, ny, nz;
    int32_t       field;
    double        h; /* grid spacing */
    const int8_t* bd;
} ngb_poisson_desc;

/* out = A u: Fixed rows copy u; Free rows (n_valid u - sum of valid
 * neighbours) / h^2 with neighbours valid inside the box. Replaces
 * LaplacianMatVec::matVec (libNeonSolver/src/linear/matvecs/LaplacianMatVec.cu:9-99). */
int ngb_laplacian_apply(const ngb_poisson_desc* desc, const void* u, void* out, void* stream);

/* Doubles of scratch a dot product of n elements needs (per-CTA partials
 * and a ticket word). */
size_t ngb_dot_scratch_doubles(int64_t n);

/* *result (device double) = sum_i a_i b_i accumulated in FP64 with a fixed
 * reduction tree (run-to-run deterministic): warp shuffles, per-CTA partials
 * in `scratch`, the last CTA to finish sums the partials in CTA order.
 * `field` selects float or double inputs. Replaces the stubbed grid dot
 * (dGrid::dot, dGrid_imp.h:254-281; ReduceKernels.cuh:7-76 compiled out). */
int ngb_dot(int64_t n, int32_t field, const void* a, const void* b, double* result, double* scratch, void* stream);

/* Flexible CG(1) vector steps with device-side scalars, so an iteration
 * needs no host round trip (no counterpart in the reference: libNeonSolver
 * has plain CG only). FP32 vectors of n elements, FP64 solution x, sums
 * accumulated as in ngb_dot. `scratch` holds ngb_fcg_scratch_doubles(n)
 * doubles; calls on one scratch must not overlap on the GPU.
 * Direction: coef = *zq / *pq_prev (zq NULL: first direction, coef 0);
 * p = z - coef p_prev and q = az - coef q_prev overwrite z and az;
 * out[0] = <p, q>, out[1] = <p, r> (device doubles). */
size_t ngb_fcg_scratch_doubles(int64_t n);
int    ngb_fcg_direction(int64_t n, void* z, void* az, const void* p_prev, const void* q_prev, const void* r, const double* zq,
                         const double* pq_prev, double* out, double* scratch, void* stream);
/* Update: alpha = pq_pr[1] / pq_pr[0]; x += alpha p, r -= alpha q; *rr = <r, r>. */
int ngb_fcg_update(int64_t n, double* x, const void* p, void* r, const void* q, const double* pq_pr, double* rr, double* scratch,
                   void* stream);

/* Allocation-free form of ngb_dot (no counterpart in the reference): for
 * callers that cannot allocate device memory where they need the reduction
 * (between launches of a stream-ordered pipeline, where cudaMalloc would
 * synchronise the device, or in a host plug-in whose device memory the host
 * application owns). Same FP64-accumulated, run-to-run deterministic result
 * as ngb_dot up to summation order; the per-CTA partials live in a fixed
 * 256 KiB array inside this library (held on every GPU that loads it until
 * exit), so n is limited to 2^28 elements (NGB_ERR_RANGE beyond). Calls no
 * cudaMalloc/cudaFree. Each call looks up the array's device address in the
 * CUDA context current on the calling thread (primary or driver-API context);
 * a call under stream capture reuses the address the last uncaptured call saw
 * in that context, so make one call in a context before capturing there. All
 * calls share the array: calls whose kernels overlap on the GPU race. */
#define NGB_DOT_NOALLOC_MAX_N (268435456LL)
int ngb_dot_noalloc(int64_t n, int32_t field, const void* a, const void* b, double* result, void* stream);

typedef struct ngb_cg_params {
    double  tol;           /* stop when |b - A x| / |b| <= tol (true residual, FP64) */
    int32_t max_iter;
    int32_t refresh_every; /* true-residual recompute period (iterative refinement), >= 1 */
    int32_t check_every;   /* iterations per captured CUDA graph between host polls, >= 1 */
    int32_t jacobi;        /* 1: Jacobi preconditioner z = r / diag(A); 0: plain CG */
} ngb_cg_params;

typedef struct ngb_cg_result {
    int32_t iterations;
    int32_t converged;
    int32_t refreshes;
    int32_t pad;
    double  rel_residual; /* last true relative residual */
    double  seconds;      /* wall time of the iteration loop */
} ngb_cg_result;

/* Bytes of device workspace ngb_cg_solve needs for this desc. */
size_t ngb_cg_workspace_bytes(const ngb_poisson_desc* desc);

/* Solves A x = b (A as ngb_laplacian_apply). Fields r, p, s and the
 * increment of x are in `desc->field` precision; every reduction, the
 * solution x (double, device, in: initial guess, out: solution) and the
 * periodic true residual b - A x are FP64 (iterative refinement). alpha,
 * beta and the stopping decision stay on the device; the iteration is
 * captured once as a CUDA graph of `check_every` iterations and the host
 * polls a 4-byte flag between graph launches. Synchronous.
 * Replaces CG_t::solve (libNeonSolver/src/linear/krylov/CG.cpp:55-156) with
 * the containers of CGContainers.cu:11-149. */
int ngb_cg_solve(const ngb_poisson_desc* desc, const void* b, double* x, void* workspace, size_t workspace_bytes,
                 const ngb_cg_params* params, ngb_cg_result* result, void* stream);

/* Measurement aid (no reference counterpart): CUDA-event time per launch of
 * the solver's two fused passes, each launched `reps` times back to back
 * from the state after x's initial residual (pass A: p = z + beta p,
 * s = A p, <p, s>; pass B: x += alpha p, r -= alpha s, <r, z>, <r, r>).
 * ms[0] = pass A, ms[1] = pass B (milliseconds per launch). Overwrites the
 * workspace and adds the timed increments to x's low part only (x itself is
 * read, not changed). Synchronous. */
int ngb_cg_time_passes(const ngb_poisson_desc* desc, const void* b, double* x, void* workspace, size_t workspace_bytes,
                       int32_t reps, float* ms, void* stream);

/* Right-hand side of the Poisson case: f = sum of 8 Gaussians
 * A_k exp(-|x - c_k|^2 / (2 sigma^2)), centres (8x3) and amplitudes from the
 * caller (see ngb_gaussian_sources), written in `field` precision. */
int ngb_poisson_rhs(const ngb_poisson_desc* desc, const double* centres, const double* amps, double sigma, void* f,
                    void* stream);

/* Deterministic sources: centres uniform in [n/8, 7n/8) per axis, amplitudes
 * uniform in [-1, 1), from std::mt19937_64(seed) 53-bit uniforms (host). */
int ngb_gaussian_sources(int32_t nx, int32_t ny, int32_t nz, uint64_t seed, double* centres, double* amps);

/* ------------------------------------------------------------------------
 * Learned preconditioner: kernels of a small 3-D U-Net (no reference
 * counterpart; the reference has no learned solver). Tensors are BF16 or FP32,
 * channels-last on an nx*ny*nz grid: element (voxel v, channel c) at v*ld + c.
 * ---------------------------------------------------------------------- */

/* 3x3x3 convolution with zero padding as an implicit GEMM on the tensor cores
 * (BF16 operands, FP32 accumulation): y[v][co] = act(sum_{t,ci} x[v+t][ci] w[co][t][ci] + bias[co]).
 * cin % 16 == 0; cout in {8, 16, 32, 48, 64}; w is [cout][27][cin] BF16
 * (t = 9(dz+1) + 3(dy+1) + (dx+1)); bias FP32 or NULL. out_f32 = 0: BF16
 * output with optional ReLU; 1: FP32 output, optionally added to y. */
int ngb_conv3d(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* w, const float* bias,
               void* y, int32_t ldy, int32_t cout, int32_t out_f32, int32_t relu, int32_t accumulate, void* stream);

/* The same convolution on the 5th-generation tensor cores (tcgen05.mma with
 * the accumulator in TMEM, operands staged by TMA; no reference counterpart).
 * Shapes it takes (ngb_conv3d_tc_supported returns 1): cin % 16 == 0,
 * cout in {16, 32, 48, 64, 96}, ldx and ldy multiples of 8, and either
 * nx % 128 == 0 or nx a divisor of 128 with ny % (128 / nx) == 0; x, y, the
 * packed weights and bias 16-byte aligned. `wpacked` is the operand image
 * written by ngb_conv3d_pack from [cout][27][cin] BF16 weights (same size).
 * Asynchronous; ngb_conv3d_tc_check(stream) synchronises the stream and
 * returns NGB_ERR_TIMEOUT if a pipeline wait of any earlier launch ran out
 * (results of that launch are then invalid). */
int ngb_conv3d_tc_supported(int32_t nx, int32_t ny, int32_t nz, int32_t ldx, int32_t cin, int32_t ldy, int32_t cout);
int ngb_conv3d_pack(int32_t cout, int32_t cin, const void* w, void* wpacked, void* stream);
int ngb_conv3d_tc(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* wpacked,
                  const float* bias, void* y, int32_t ldy, int32_t cout, int32_t out_f32, int32_t relu, int32_t accumulate,
                  void* stream);
int ngb_conv3d_tc_check(void* stream);
/* Self-test of the kernels' bounded waits: one thread polls, `limit` times at
 * most (1 .. 2^20), an mbarrier that nothing arrives on, with no copy or MMA
 * in flight. The wait runs out and raises the same error flag a pipeline
 * wait of ngb_conv3d_tc does; returns NGB_OK when it gave up as designed (the
 * next ngb_conv3d_tc_check then returns NGB_ERR_TIMEOUT and clears the flag). */
int ngb_conv3d_tc_wait_selftest(int32_t limit, void* stream);

/* dw[co][t][ci] += sum_v dy[v][co] x[v+t][ci] (BF16 inputs, FP32 dw). Runs
 * on the tcgen05 tensor cores where ngb_conv3d_bwd_weight_tc_supported
 * allows, on the mma.sync kernel elsewhere. */
int ngb_conv3d_bwd_weight(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* dy, int32_t lddy,
                          int32_t cout, float* dw, void* stream);
/* The tcgen05 form alone: an implicit GEMM per group of 128 / cin taps
 * (M = 128 rows (tap, ci), N = cout, K = voxels, FP32 accumulators in TMEM),
 * operands gathered and transposed into shared memory by the CTA; the CTAs'
 * partial sums over voxel ranges go to a scratch array (allocated on first
 * use per device, grown on demand) and are added to dw in a fixed order, so
 * repeated calls give the same bits. Shapes: nx % 8 == 0, the
 * voxel count a multiple of 64, cin % 8 == 0 and <= 128, cout in
 * {16, 32, 64}, ldx / lddy multiples of 8, x and dy 16-byte aligned. */
int ngb_conv3d_bwd_weight_tc_supported(int32_t nx, int32_t ny, int32_t nz, int32_t ldx, int32_t cin, int32_t lddy, int32_t cout);
int ngb_conv3d_bwd_weight_tc(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* dy,
                             int32_t lddy, int32_t cout, float* dw, void* stream);
/* The mma.sync form alone (any shape ngb_conv3d_bwd_weight takes: cin % 16 == 0, cout % 8 == 0, cout <= 64). */
int ngb_conv3d_bwd_weight_mma(int32_t nx, int32_t ny, int32_t nz, const void* x, int32_t ldx, int32_t cin, const void* dy,
                              int32_t lddy, int32_t cout, float* dw, void* stream);

/* out = BF16(dy * (y > 0)) (ReLU backward; y NULL: no mask). */
int ngb_relu_bwd(int64_t V, int32_t C, const float* dy, int32_t lddy, const void* y, int32_t ldy, void* out, int32_t ldo, void* stream);

/* 2x2x2 average pooling (BF16) of an even fine grid and its adjoint (FP32, optionally accumulated). */
int ngb_pool2(int32_t nx, int32_t ny, int32_t nz, int32_t C, const void* x, int32_t ldx, void* y, int32_t ldy, void* stream);
int ngb_pool2_bwd(int32_t nx, int32_t ny, int32_t nz, int32_t C, const float* dy, int32_t lddy, float* dx, int32_t lddx,
                  int32_t accumulate, void* stream);

/* Nearest 2x upsampling to the fine grid (BF16) and its adjoint (FP32). */
int ngb_up2(int32_t nx, int32_t ny, int32_t nz, int32_t C, const void* x, int32_t ldx, void* y, int32_t ldy, void* stream);
int ngb_up2_bwd(int32_t nx, int32_t ny, int32_t nz, int32_t C, const float* dy, int32_t lddy, float* dx, int32_t lddx, void* stream);

/* Adam step on FP32 master weights (bias-corrected with `step`), writing the
 * BF16 copy `pb` if non-NULL. */
int ngb_adam(int64_t n, float* p, const float* g, float* m, float* s, float lr, float b1, float b2, float eps, int32_t step, void* pb,
             void* stream);

/* wt[ci][26 - t][co] = BF16(w[co][t][ci]): weights of the backward-data convolution. */
int ngb_flip_weights(int32_t cout, int32_t cin, const float* w, void* wt, void* stream);

/* Network input and output with the scale kept on the device (no host
 * round trip). `rr` is a device double holding |r|^2 (ngb_dot), sigma =
 * sqrt(rr / V) (1 for a zero field). Input: channel 0 of the channels-last
 * BF16 tensor in0 (row stride ld) = bf16(r / sigma); the other channels are
 * left as they are. Output: e = scale * sigma * out[v * ld] on the interior
 * of the nx*ny*nz box, 0 on its faces. */
int ngb_unet_input(int64_t V, const float* r, const double* rr, void* in0, int32_t ld, void* stream);
int ngb_unet_output(int32_t nx, int32_t ny, int32_t nz, const float* out, int32_t ld, const double* rr, double scale, float* e,
                    void* stream);

/* e *= num / den when both device doubles are positive, else e = 0 (the
 * energy-minimising step of a correction e: num = <e, r>, den = <e, A e>). */
int ngb_scale_by_ratio(int64_t n, float* e, const double* num, const double* den, void* stream);

/* ------------------------------------------------------------------------
 * Multilevel learned preconditioner: smoothing and grid transfer between
 * vertex-centred levels (no reference counterpart; libNeonSolver has CG
 * only). FP32 fields on the box-face Dirichlet problem (desc->bd == NULL,
 * desc->field NGB_STORE_F32); A is the operator of ngb_laplacian_apply with
 * spacing desc->h. Coarse node I sits on fine node 2I: a fine grid of even
 * dims n has the coarse grid n/2 with spacing 2h. Face nodes of every level
 * are Fixed and written as 0.
 * ---------------------------------------------------------------------- */

/* Damped Jacobi on the Free nodes: out = u + omega h^2/6 (r - A u). With u
 * NULL, out is the result of two sweeps from u = 0 in one stencil pass over
 * r (2 c r - c^2 A r, c = omega h^2/6; r must be 0 on the face nodes). */
int ngb_mg_jacobi(const ngb_poisson_desc* desc, const void* u, const void* r, void* out, double omega, void* stream);

/* out = A u on the Free nodes, 0 on the face nodes. */
int ngb_mg_apply(const ngb_poisson_desc* desc, const void* u, void* out, void* stream);

/* out = r - A u on the Free nodes (u NULL: u = 0). */
int ngb_mg_residual(const ngb_poisson_desc* desc, const void* u, const void* r, void* out, void* stream);

/* Full-weighting restriction to the coarse grid (dims/2): rc(I) = scale *
 * sum_a w_a res(2I + a), w = (1/4, 1/2, 1/4) per axis, on coarse interior
 * nodes; fine dims even and >= 6. */
int ngb_mg_restrict(const ngb_poisson_desc* fine, const void* res, void* rc, double scale, void* stream);

/* u += P ec on the fine Free nodes, P the trilinear interpolation from the
 * coarse grid (dims/2) that ngb_mg_restrict's weights are the transpose of. */
int ngb_mg_prolong_add(const ngb_poisson_desc* fine, const void* ec, void* u, void* stream);

/* ------------------------------------------------------------------------
 * Learned-preconditioner Poisson solver (no reference counterpart:
 * libNeonSolver has plain CG only, CG.h:70-76; this is its learned sibling
 * with the same solve(b, x) -> result shape). FCG(1) on A x = b for the
 * zero-Dirichlet n^3 box (A as ngb_laplacian_apply, h = 1), preconditioned
 * by a V-cycle of `levels` damped-Jacobi levels whose coarsest-level solve is
 * the 3-level U-Net (16/32/64 channels, BF16 tensor-core convolutions) on the
 * (n / 2^levels)^3 grid; x accumulates in FP64, the true residual b - A x is
 * recomputed in FP64 every refresh_every iterations, and Jacobi-PCG
 * (ngb_cg_solve) takes over from x when that residual fails to halve over
 * `stall` iterations or the iteration breaks down. The solver owns its
 * device buffers. */
typedef struct ngb_learned_solver ngb_learned_solver;

typedef struct ngb_learned_params {
    double  tol;           /* stop when |b - A x| / |b| <= tol (FP64 true residual) */
    int32_t max_iter;      /* FCG iterations before giving up (fallback excluded) */
    int32_t refresh_every; /* true-residual period, >= 1 (10 in the benchmark) */
    int32_t stall;         /* fallback when the true residual does not halve over this many iterations */
    int32_t fallback;      /* 1: Jacobi-PCG takes over on stagnation or breakdown */
} ngb_learned_params;

typedef struct ngb_learned_result {
    int32_t iterations;          /* FCG iterations */
    int32_t fallback;            /* 1 if Jacobi-PCG took over */
    int32_t fallback_iterations; /* its iterations */
    int32_t converged;
    double  rel_residual;        /* final true relative residual */
    double  seconds;             /* wall time of the solve */
} ngb_learned_result;

/* Number of FP32 weights of the network (10 layers [cout][27][cin] in the
 * order c0a c0b c1a c1b c2a c2b c1c c1d c0c c0d). */
int64_t ngb_unet_weight_count(void);
/* Weight file: "NGBUNET1", version 1, 10 layers of (cout, cin, BF16 values).
 * write rounds FP32 to BF16 (nearest even); read returns exact FP32 values. */
int ngb_unet_write_weights(const char* path, const float* weights, int64_t count);
int ngb_unet_read_weights(const char* path, float* weights, int64_t count);

/* Creates the solver for an n^3 grid: n a multiple of 2^levels, the coarsest
 * grid n / 2^levels >= 8 and a multiple of 4 (two poolings); weights: host
 * FP32 array of ngb_unet_weight_count() values, or NULL with count 0 for the
 * same V-cycle without the network (the level above the coarsest gets no
 * correction). Allocates device memory. */
int ngb_learned_create(int32_t n, int32_t levels, const float* weights, int64_t count, ngb_learned_solver** solver);
int ngb_learned_destroy(ngb_learned_solver* solver);
/* z = M(r): one application of the preconditioner (FP32 n^3 fields). */
int ngb_learned_precondition(ngb_learned_solver* solver, const float* r, float* z, void* stream);
/* Solves A x = b (b FP32, zero on the faces; x FP64 initial guess and
 * solution). Synchronous; reads one double from the device per iteration. */
int ngb_learned_solve(ngb_learned_solver* solver, const float* b, double* x, const ngb_learned_params* params,
                      ngb_learned_result* result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NEON_GB300_H */
