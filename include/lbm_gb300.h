/*
 * lbm_gb300.h -- C ABI of the GB300 (sm_103a) collide-stream library.
 *
 * Drop-in boundary for lbmminiapp's hot path: the BGK collision with Guo
 * forcing fused with streaming, for D3Q19 and D3Q27, under AA (one buffer,
 * even/odd steps) and AB (two buffers, push or pull) propagation, on an SOA
 * population layout with half-way bounce-back from a solid mask.  On one GPU
 * the reference's MPI halo exchange (src/Communication.cpp:379-481, a no-op on
 * one rank) becomes the periodic wrap and mask bounce-back computed inside
 * the kernels.
 *
 * Plain C types only: no CUDA, torch or C++ types cross this boundary.  Every
 * call returns an lbm_status; no exception crosses it.  One handle must not be
 * used from two host threads at once; separate handles are independent.
 *
 * Array conventions
 *   cell index       c = x + nx*(y + ny*z)          (x fastest)
 *   host arrays      dense over all nx*ny*nz cells; per-direction and vector
 *                    arrays planar: [component][cell]
 *   directions       the reference's order and opposite table
 *                    (src/lattices/LatticeD3Q19.cpp:5-88,
 *                    src/lattices/LatticeD3Q27.cpp:5-120)
 *   raw layout       slot contents as the reference stores them: AA at even
 *                    time holds direction s in slot opp(s)
 *                    (src/propagation/PropagationAA.cpp:104-116); AB pull
 *                    holds post-collision values not yet streamed
 *   logical layout   direction s of each cell, post-stream, pre-collision
 *   solid cells      read back as NaN
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lbm_status {
   LBM_OK = 0,
   LBM_ERR_INVALID_ARGUMENT = 1,
   LBM_ERR_OUT_OF_MEMORY = 2, /* device allocation failed or over max_device_bytes */
   LBM_ERR_CUDA = 3,          /* CUDA runtime error; see lbm_last_error */
   LBM_ERR_DIVERGED = 4,      /* NaN/Inf found by a conservation reduction */
   LBM_ERR_UNSUPPORTED = 5,   /* valid request the library does not provide */
   LBM_ERR_STATE = 6          /* call not valid in the handle's current state */
} lbm_status;

/* Propagation pattern: the reference input-file key propPattern
 * (src/Parameters.cpp:56-59; AB = 0, AA = 1). */
enum { LBM_PATTERN_AB = 0, LBM_PATTERN_AA = 1 };

/* Population storage.  F64 stores f as the reference's Pdf=double buffer;
 * F32/BF16/F16 store the shifted value f - w (F16 scaled by 2^15). */
enum { LBM_STORE_F64 = 0, LBM_STORE_F32 = 1, LBM_STORE_BF16 = 2, LBM_STORE_F16 = 3 };

/* Collision arithmetic.  AUTO = F64X for F64 storage, F32 otherwise.
 *   F64  IEEE double with the reference Base kernels' operation order and no
 *        FMA contraction (bit-identical to the reference CPU build).
 *   F64X double-precision result computed with FP32-pair arithmetic
 *        (about 47 significant bits; GB300's FP64 pipe is 1/64 of its FP32
 *        rate); stores FP64.
 *   F32  single precision on shifted populations. */
enum { LBM_ARITH_AUTO = 0, LBM_ARITH_F64 = 1, LBM_ARITH_F64X = 2, LBM_ARITH_F32 = 3 };

enum { LBM_LAYOUT_RAW = 0, LBM_LAYOUT_LOGICAL = 1 };

typedef struct lbm_config {
   int lattice;       /* 19 or 27 (_LATTICESIZE_, src/Parameters.hh:6-8) */
   int prop_pattern;  /* LBM_PATTERN_AB or LBM_PATTERN_AA */
   int pull;          /* AB only: 0 push, 1 pull (input key "pull") */
   int unroll;        /* 1: weight the Q19 AA rest population's forcing term
                         with 1/36 as KernelAA_SOA_Unroll does
                         (src/kernels/KernelAA_SOA_Unroll.cpp:556,770) */
   int nx, ny, nz;
   int periodic[3];   /* per axis; a non-periodic face bounces back */
   double omega;      /* _OMEGA_ (src/Parameters.hh:26-28) */
   double force[3];   /* uniform body force; the reference's _GRAVITY_ is force[0] */
   int storage;       /* LBM_STORE_* */
   int arithmetic;    /* LBM_ARITH_* */
   int device;        /* CUDA device ordinal */
   int compact;       /* 1: keep populations for fluid cells only (compact
                         fluid-only storage; AA with F32/BF16/F16 storage),
                         for media with many solid cells.  Host-facing arrays
                         stay dense; no per-cell fields.  0: dense grid */
   uint64_t max_device_bytes; /* 0 = no cap; else creation fails with OOM above it */
} lbm_config;

typedef struct lbm_info {
   int64_t ncell;          /* nx*ny*nz */
   int64_t nfluid;         /* cells not marked solid (MLUPS counts these) */
   int64_t time_step;      /* steps taken since the last initialisation */
   int64_t plane_stride;   /* elements between direction planes of a buffer */
   uint64_t buffer_bytes;  /* bytes of one population buffer */
   uint64_t device_bytes;  /* device memory held by the handle */
   int bytes_per_update;   /* 2*Q*sizeof(stored population): algorithmic bytes */
   int lattice;
   int storage;
   int arithmetic;         /* resolved (never AUTO) */
} lbm_info;

typedef struct lbm_handle lbm_handle;

/* ---- lifetime (replaces Propagation{AA,AB}::setup and the Kernel*::setup
 *      table uploads: src/propagation/PropagationAA.cpp:10-57,
 *      src/propagation/PropagationAB.cpp:16-88, src/kernels/KernelAA.hh:23) */
lbm_status lbm_config_default(lbm_config* cfg);
lbm_status lbm_create(const lbm_config* cfg, lbm_handle** out);
void lbm_destroy(lbm_handle* h);
const char* lbm_last_error(const lbm_handle* h); /* never NULL */
const char* lbm_status_string(lbm_status s);
lbm_status lbm_get_info(const lbm_handle* h, lbm_info* info);
/* cudaStream_t passed as void*; NULL = the legacy default stream.  A handle's
 * step kernels share its tile counters (zero between launches), so its steps
 * run in one stream order: after switching streams, order the new stream after
 * the old one's last step (an event) before the next step. */
lbm_status lbm_set_stream(lbm_handle* h, void* stream);
lbm_status lbm_synchronize(lbm_handle* h);

/* ---- geometry (replaces Geometry::setupGrid / GeometryAAAB::setupAdjacency:
 *      src/geometries/Geometry.cpp:100-151, src/geometries/GeometryAAAB.cpp:18-124;
 *      the adjacency list becomes in-kernel index arithmetic plus one 32-bit
 *      link word per cell) */
/* solid: host, ncell bytes, nonzero = solid. NULL = no solid cells. */
lbm_status lbm_set_solid(lbm_handle* h, const uint8_t* solid);
/* Cylinder of the reference (src/geometries/Geometry.cpp:59-71,112-140):
 * writes nx,ny,nz for simulationSize into dims[3] and, when solid != NULL, the
 * mask (dims product bytes). */
lbm_status lbm_geometry_cylinder(double simulation_size, int dims[3], uint8_t* solid);

/* ---- optional per-cell fields (no reference counterpart) */
/* F(x) = cfg.force + field(x); host, planar [3][ncell]; NULL removes. */
lbm_status lbm_set_force_field(lbm_handle* h, const double* field);
/* Partial bounce-back solid fraction s(x) in [0,1]; NULL removes. */
lbm_status lbm_set_porosity(lbm_handle* h, const double* porosity);

/* ---- state (replaces Propagation{AA,AB}::initialize:
 *      src/propagation/PropagationAA.cpp:60-123, PropagationAB.cpp:91-152) */
/* f = equilibrium(rho, u); rho NULL -> 1, u NULL -> 0 (rest state f = w as in
 * the reference).  Host arrays.  Resets time_step to 0. */
lbm_status lbm_init_equilibrium(lbm_handle* h, const double* rho, const double* u);
/* Host populations [Q][ncell] in the given layout.  Resets time_step to 0
 * for LOGICAL; RAW keeps it. */
lbm_status lbm_set_populations(lbm_handle* h, const double* f, int layout);
lbm_status lbm_get_populations(lbm_handle* h, double* f, int layout);

/* ---- time loop (replaces Propagation{AA,AB}::run:
 *      src/propagation/PropagationAA.cpp:126-215,
 *      src/propagation/PropagationAB.cpp:155-219): one launch per step,
 *      asynchronous on the handle's stream. */
lbm_status lbm_step(lbm_handle* h, int nsteps);

/* ---- readouts */
/* rho[ncell], u[3][ncell] = sum(c f)/rho without the F/2 shift, with the
 * reference's getRho/getVelocity semantics (PropagationAA.cpp:218-327,
 * PropagationAB.cpp:222-281). */
lbm_status lbm_get_macros(lbm_handle* h, double* rho, double* u);
/* FP64 sums over fluid cells of rho and rho*u (no F/2 shift) from the logical
 * populations: out[0]=mass, out[1..3]=momentum.  Cells whose populations all
 * lie in [2^-32, 1) are summed exactly (128-bit fixed point) and the totals
 * rounded once, so they do not depend on launch shapes; other cells are
 * summed in FP64.  LBM_ERR_DIVERGED when a sum is not finite.  No reference
 * counterpart. */
lbm_status lbm_reduce_conserved(lbm_handle* h, double out[4]);

/* ---- kernel-level entry points on caller-owned device buffers.
 * dstrb/src/tgt: device pointers to buffers of info.buffer_bytes in the
 * handle's storage type and raw layout (planar, info.plane_stride elements per
 * direction).  start/count: a range of cell indices; solid cells in it are
 * skipped.  The handle's own buffers are not touched. */
/* KernelAA::timestepEvenForce(Pdf* dstrb, int startIdx, int countIdx)
 * (src/kernels/KernelAA.hh:28) */
lbm_status lbm_timestep_even_force(lbm_handle* h, void* dstrb, int64_t start, int64_t count);
/* KernelAA::timestepOddForce (src/kernels/KernelAA.hh:29) */
lbm_status lbm_timestep_odd_force(lbm_handle* h, void* dstrb, int64_t start, int64_t count);
/* KernelAB::timestepForce(Pdf* src, Pdf* tgt, int startIdx, int countIdx)
 * (src/kernels/KernelAB.hh:28); push or pull per cfg.pull */
lbm_status lbm_timestep_force(lbm_handle* h, const void* src, void* tgt, int64_t start,
                              int64_t count);
/* Device pointer of the handle's current population buffer (the one
 * lbm_get_populations reads). */
lbm_status lbm_population_buffer(lbm_handle* h, void** dev_ptr);

/* ---- adjoint (no reference counterpart).  Differentiates a rollout of
 * AB-push steps (prop_pattern AB, pull 0: the stored buffer is then the
 * pre-collision state f^t) with respect to the per-cell force field and
 * porosity.  All arrays below are device memory, FP64, planar with
 * info.plane_stride elements per component.  The host drives checkpointed
 * recomputation (lbmminiapp_gb300/adjoint.py). */
enum { LBM_LOSS_NONE = 0, LBM_LOSS_VELOCITY = 1, LBM_LOSS_ENERGY = 2 };
/* Copy the handle's current population buffer to (to_handle = 0) or from
 * (to_handle = 1) a caller device buffer of info.buffer_bytes. */
lbm_status lbm_copy_state(lbm_handle* h, void* dev, int to_handle);
/* Per-cell force field [3][plane] and porosity [plane] from device memory;
 * NULL removes the field. */
lbm_status lbm_set_fields_device(lbm_handle* h, const double* force_field, const double* porosity);
/* Loss of a state (NULL = the handle's current one):
 *   LBM_LOSS_VELOCITY: time_weight * sum_x W(x).u(x), W [3][plane]
 *   LBM_LOSS_ENERGY:   time_weight * sum_x W(x) rho |u|^2 / 2, W [plane]
 * with u = (sum c f + F/2)/rho.  FP64; *out_host receives the value. */
lbm_status lbm_loss(lbm_handle* h, const void* state, int loss_kind, const double* weight, double time_weight,
                    double* out_host);
/* One adjoint step: lam = dL/df^t from lam_next = dL/df^{t+1} and the state
 * f^t (a buffer in the handle's storage); accumulates into grad_force
 * [3][plane] and grad_porosity [plane] (either may be NULL).  collide = 0
 * keeps only the loss term (the final state of a rollout); the loss term is
 * added when loss_kind != LBM_LOSS_NONE. */
lbm_status lbm_adjoint_step(lbm_handle* h, const void* state, const double* lam_next, double* lam, int collide,
                            int loss_kind, const double* weight, double time_weight, double* grad_force,
                            double* grad_porosity);
/* lbm_adjoint_step with lam, lam_next and the arithmetic in FP32 (on the
 * deviations f - w); grad_force and grad_porosity are still FP64 accumulators.
 * For rollouts whose forward runs in reduced-precision storage. */
lbm_status lbm_adjoint_step_f32(lbm_handle* h, const void* state, const float* lam_next, float* lam, int collide,
                                int loss_kind, const double* weight, double time_weight, double* grad_force,
                                double* grad_porosity);

/* ---- compact fluid-only layout (the reference's own buffers and adjacency).
 * The reference keeps populations only for fluid points, direction s of fluid
 * point i at dstrb[nFluid*s + i], and streams through the int32 adjacency list
 * of GeometryAAAB::setupAdjacency (src/geometries/GeometryAAAB.cpp:18-124):
 * adjacency[nFluid*s + i] is the element index of slot s at the neighbour
 * x - c_s (AA, AB pull) or x + c_s (AB push), or nFluid*opp(s) + i for a wall.
 * A sparse handle holds a device copy of that list and runs the reference's
 * kernel steps on caller-owned device buffers in that layout, in any fluid
 * order.  cfg: lattice, prop_pattern, pull, unroll, omega, force, arithmetic
 * (AUTO/F64X or F64), device and max_device_bytes are used; storage must be
 * LBM_STORE_F64; the grid fields are ignored.  Q * nfluid must stay below
 * 2^31 (the reference's int32 indices); every adjacency entry must lie in
 * [0, Q * nfluid).  Steps run asynchronously on the handle's stream. */
typedef struct lbm_sparse_handle lbm_sparse_handle;
/* GeometryAAAB::setupAdjacency's result as the handle's streaming map;
 * adjacency: host, [Q][nfluid] int32. */
lbm_status lbm_sparse_create(const lbm_config* cfg, int64_t nfluid, const int32_t* adjacency,
                             lbm_sparse_handle** out);
void lbm_sparse_destroy(lbm_sparse_handle* h);
const char* lbm_sparse_last_error(const lbm_sparse_handle* h); /* never NULL */
/* As lbm_set_stream: the handle's steps share its tile counters and run in one
 * stream order. */
lbm_status lbm_sparse_set_stream(lbm_sparse_handle* h, void* stream);
/* KernelAA::timestepEvenForce(Pdf* dstrb, int startIdx, int countIdx)
 * (src/kernels/KernelAA.hh:28) on a compact device buffer of Q*nfluid doubles */
lbm_status lbm_sparse_timestep_even_force(lbm_sparse_handle* h, double* dstrb, int64_t start, int64_t count);
/* KernelAA::timestepOddForce (src/kernels/KernelAA.hh:29) */
lbm_status lbm_sparse_timestep_odd_force(lbm_sparse_handle* h, double* dstrb, int64_t start, int64_t count);
/* KernelAB::timestepForce(Pdf* src, Pdf* tgt, int startIdx, int countIdx)
 * (src/kernels/KernelAB.hh:28); push or pull per cfg.pull */
lbm_status lbm_sparse_timestep_force(lbm_sparse_handle* h, const double* src, double* tgt, int64_t start,
                                     int64_t count);

/* ---- allocation-free conservation reduction.  No counterpart in the
 * reference.  For callers that cannot allocate device memory while they run
 * (hosts that give every device byte to their own pool at start-up, drivers
 * that must not allocate inside their time loop) and therefore cannot create a
 * handle.  Everything is caller-owned device memory: dstrb (a population
 * buffer in the raw layout of the given storage, plane_stride elements per
 * direction), solid (ncell bytes, nonzero = solid; NULL = none) and out (4
 * doubles: mass, momentum x/y/z, as lbm_reduce_conserved).  periodic is a
 * host array of 3 flags.  readout: 0 = slot s holds direction s (AB push),
 * 1 = AA at even time (slot opp(s)), 2 = pull gather (AA at odd time, AB
 * pull).  Asynchronous on `stream` (cudaStream_t as void*, NULL = legacy
 * default stream), on the current device; out is not checked for NaN/Inf.
 * Calls no cudaMalloc: the per-block partial sums live in a static device
 * array of 384 KiB that every GPU loading the library keeps until exit, so at
 * most 2^28 (268,435,456) cells are accepted; larger grids return
 * LBM_ERR_INVALID_ARGUMENT.  The first call on each device looks the array's
 * address up (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  The address is kept for the life of the
 * process, so calls must run in the device's primary context (the CUDA
 * runtime's own) and the device must not be reset (cudaDeviceReset) between
 * calls.  All calls share the array: calls that overlap on the GPU race. */
lbm_status lbm_reduce_conserved_noalloc(int lattice, int storage, int nx, int ny, int nz,
                                        int64_t plane_stride, const void* dstrb, const uint8_t* solid,
                                        const int periodic[3], int readout, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif
