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

/* ------------------------------------------------------------------------
 * Lattice-Boltzmann populations
 * ---------------------------------------------------------------------- */

/* How populations are held in HBM. The *_OFF forms hold g_q = f_q - w_q. */
typedef enum {
    NGB_STORE_F64 = 0,
    NGB_STORE_F32 = 1,
    NGB_STORE_F16OFF = 2,
    NGB_STORE_BF16OFF = 3
} ngb_storage;

/* Cell classification, values of benchmarks/lbm-lid-driven-cavity-flow/src/CellType.h:5-11
 * plus OUTLET (zero-gradient outflow node, new). */
typedef enum {
    NGB_CELL_BOUNCEBACK = 0,
    NGB_CELL_MOVINGWALL = 1,
    NGB_CELL_BULK = 2,
    NGB_CELL_UNDEFINED = 3,
    NGB_CELL_OUTLET = 4
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
 * per (desc, pointers) and replayed. Replaces the host loop of
 * RunCavityTwoPop.cu:257-273 over LbmIterationD3Q19::run (LbmIteration.h:56-61). */
int ngb_lbm_dense_run(const ngb_lbm_dense_desc* desc, void* fa, void* fb, const uint32_t* flags, int32_t nsteps, void* stream);

/* Host-buffer form of ngb_lbm_dense_run for callers whose populations live
 * in host memory: copies host_in (pinned or pageable, q*plane_stride
 * elements) into fa, runs nsteps, and copies the newest populations back to
 * host_out; fa/fb are caller-provided device buffers. Stream-ordered; the
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

#ifdef __cplusplus
}
#endif

#endif /* NEON_GB300_H */
