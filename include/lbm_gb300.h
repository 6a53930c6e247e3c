/*
 * lbm_gb300.h -- C ABI of the GB300 (sm_103a) Allen-Cahn phase-field lattice
 * Boltzmann time step (D3Q19, conservative Allen-Cahn phase field + Fakhari
 * pressure-velocity hydrodynamics, geometric-amplification wetting, volume
 * penalisation, global phi-mass correction).
 *
 * One opaque handle owns one grid's device state.  All entry points return 0
 * on success or a negative LBM_E* code; lbm_last_error() gives a message for
 * the calling thread.  No exception crosses the ABI.  Pointers are plain host
 * or device addresses as documented per argument; streams are cudaStream_t
 * passed as void* (NULL = legacy default stream).
 *
 * Each entry point replaces one part of the reference's Python surface
 * (pytorch-lbm, file:line cited per function).  Layout of every field is the
 * reference's: C-contiguous (nx, ny, nz), z fastest; vectors (3, nx, ny, nz);
 * populations (19, nx, ny, nz) in the D3Q19 order of lbm/lattice.py:70-81.
 * A grid with nz == 1 is 2-D, as in the reference (lbm/fe_config.py:157):
 * D2Q9 populations (9, nx, ny) in the order of lbm/lattice.py:46-55, vectors
 * (2, nx, ny), wall normals (2, nx, ny); "N" below is nx*ny*nz either way.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define LBM_OK 0
#define LBM_E_ARG -1        /* invalid argument / size / null pointer         */
#define LBM_E_CUDA -2       /* a CUDA runtime call failed                     */
#define LBM_E_STATE -3      /* call out of order (e.g. step before init)      */
#define LBM_E_UNSUPPORTED -4

/* Precision of the state and of the collision arithmetic. */
#define LBM_F32 0           /* float populations, float arithmetic            */
#define LBM_F64 1           /* double populations, double arithmetic          */
#define LBM_F16 2           /* half populations stored as deviations from the
                               rest-state equilibria (f: F/w - phi of the
                               reading node, g: G/w), float arithmetic and
                               fields, double global sums                   */

/* Element type of a caller array. */
#define LBM_DT_NONE 0
#define LBM_DT_F32 1
#define LBM_DT_F64 2

/* stab_mode values (lbm/fe_ac_solver.py:433-438). */
#define LBM_STAB_FAKHARI 0  /* F = F_s + F_p + F_m + F_body                   */
#define LBM_STAB_LIANG 1    /* F = F_s + F_p + F_body                         */
#define LBM_STAB_NONE 2     /* F = F_s + F_body                               */

/* interface_mode values (lbm/fe_ac_solver.py:76, 457-486). */
#define LBM_IFACE_ALLEN_CAHN 0      /* conservative Allen-Cahn sharpening source   */
#define LBM_IFACE_CAHN_HILLIARD 1   /* source M (grad mu - grad phi) tau/(tau-1/2) */

/* Field selection bits for lbm_get_fields. */
#define LBM_FIELD_PHI 1u
#define LBM_FIELD_RHO 2u
#define LBM_FIELD_U 4u
#define LBM_FIELD_P 8u      /* P = sum(g)                                     */
#define LBM_FIELD_PRESS 16u /* p = P cs^2 (rho cs^2 right after init)         */
#define LBM_FIELD_MU 32u

/* Status flag bits (lbm_status). */
#define LBM_STATUS_NAN 1u        /* sum(phi) was NaN/Inf in some step         */
#define LBM_STATUS_MASS_LOW 2u   /* sum(phi) <= 1e-6: correction skipped      */

/*
 * Physical and model parameters.  Field meanings and defaults are those of
 * FEConfig (lbm/fe_config.py:27-150, already derived: beta, kappa, phi_c) and
 * of the AllenCahnSolver constructor (lbm/fe_ac_solver.py:54-58).
 */
typedef struct LbmParams {
    double rho_l, rho_g, sigma, xi, beta, kappa, phi_c;
    double tau_l, tau_g, tau_h;   /* tau_f = tau_h if tau_h > 0 else tau_l    */
    double theta_eq;              /* degrees; 90 disables wetting             */
    double g_force[3];
    double boundary_relax;        /* default 0.3                              */
    double sharpen_reduce;        /* default 0.8                              */
    double mu_wall_scale;         /* default 1.0                              */
    double geo_amplification;     /* scalar alpha_geo; default 1.0            */
    double ac_scale;              /* default 1.0                              */
    double ghost_scale;           /* <= 0: automatic (3 if |theta-90|>60 else 2) */
    int32_t stab_mode;            /* LBM_STAB_*                               */
    int32_t geometric_wetting;    /* 0/1                                      */
    int32_t interface_mode;       /* LBM_IFACE_*; default Allen-Cahn          */
    int32_t direct_wetting;       /* 0/1: cubic-wall-energy boundary phi      */
    double mu_drive;              /* >= 0; default 0 (Allen-Cahn mode only)   */
} LbmParams;

typedef struct LbmHandle LbmHandle;

/* Allocate the device state of one nx*ny*nz grid on the current CUDA device.
 * Replaces AllenCahnSolver.__init__ (lbm/fe_ac_solver.py:54-191).
 * nz == 1 makes a 2-D D2Q9 grid (the reference's 2-D path): LBM_F32 or
 * LBM_F64 only, stepped by its own per-node kernels (no fused tiles, no
 * autotuning, no batches: LBM_E_UNSUPPORTED).  3-D
 * grids need every extent >= 2.  The interface sources that need
 * the gradient of the chemical potential (interface_mode Cahn-Hilliard,
 * mu_drive > 0) add a chemical-potential pass to every step, run on LBM_F32
 * and LBM_F64 grids (LBM_E_UNSUPPORTED with LBM_F16), with the two-kernel
 * step only (no fused tile kernel) and one grid at a time (not in batches). */
int lbm_create(const LbmParams* params, int64_t nx, int64_t ny, int64_t nz,
               int precision, LbmHandle** out);

/* Free the handle.  Waits for the device's queued work (as cudaFree does),
 * then returns the grid's state arrays to the process's cache of device
 * blocks, from which lbm_create takes blocks of a fitting size (at most 1/8
 * larger, same device) before it allocates; past the cache's limit the
 * blocks cached longest are freed to make room.  The reference frees its tensors through PyTorch's caching
 * allocator, which keeps them likewise. */
int lbm_destroy(LbmHandle* h);

/* The cache of state arrays: its limit in bytes (default 16 GiB; 0 frees
 * every cached block and disables caching), freeing every cached block
 * (`freed_bytes` may be NULL), and the bytes it holds.  lbm_create also
 * empties it and retries when cudaMalloc runs out of memory.  No reference
 * counterpart (torch.cuda.empty_cache for the reference's tensors). */
int lbm_cache_limit(uint64_t bytes);
int lbm_cache_trim(uint64_t* freed_bytes);
int lbm_cache_bytes(uint64_t* cached_bytes);

/* Solid mask (host, N bytes, nonzero = solid) and optional solid fraction
 * (host, N elements of fraction_dtype, or NULL with LBM_DT_NONE).  Computes
 * on the device, bit-exact with the reference: partial-solid nodes and their
 * penalisation fraction, wetting boundary nodes, wall normals (smooth from the
 * fraction gradient, else discrete), near-wall distance and weight, the
 * top-surface flag and the node-class table.  Replaces AllenCahnSolver.set_solid
 * (lbm/fe_ac_solver.py:193-237) and ConningtonLeeWetting.__init__ /
 * _precompute_* (lbm/fe_wetting.py:39-367).  Synchronous. */
int lbm_set_geometry(LbmHandle* h, const uint8_t* solid, const void* fraction,
                     int fraction_dtype);

/* As lbm_set_geometry with the solid mask and the fraction in device memory
 * (N bytes and N elements of fraction_dtype), asynchronous on `stream`; both
 * must stay valid until the work queued on `stream` has run.  Replaces the
 * same reference code as lbm_set_geometry. */
int lbm_set_geometry_device(LbmHandle* h, const uint8_t* solid, const void* fraction,
                            int fraction_dtype, void* stream);

/* Per-node geometric amplification field alpha (host, N elements of
 * alpha_dtype, LBM_DT_F32 or LBM_DT_F64), used in place of the scalar
 * params.geo_amplification: at each wetting boundary node the contact-angle
 * correction is amplified by that node's alpha where alpha > 1 and left
 * un-amplified elsewhere.  The field is rounded to the compute type, as the
 * reference casts it.  alpha = NULL (with LBM_DT_NONE) returns to the scalar.
 * Allocates N compute-type elements on the device (not counted by
 * lbm_footprint); synchronises the device.  Replaces a tensor-valued
 * geo_amplification (lbm/fe_wetting.py:501-512, lbm/fe_ac_solver.py:83). */
int lbm_set_amplification(LbmHandle* h, const void* alpha, int alpha_dtype);

/* Initial phase field phi (N elements) and optional velocity u (3N elements,
 * 2N on a 2-D grid; NULL = zero), of element type src_dtype, in host memory (on_device = 0) or
 * device memory (on_device = 1).  Sets f = f_eq(phi, u), g = g_eq(0, u) and
 * the phi-mass reference.  Replaces AllenCahnSolver.init_fields
 * (lbm/fe_ac_solver.py:239-261).  Asynchronous on `stream` for device
 * inputs.  Host inputs may be released when the call returns: where the
 * device reads pageable host memory in place (cudaDevAttrPageableMemoryAccess,
 * a Grace host), the kernel reads them without a staging copy and the call
 * waits for it; elsewhere, or with LBM_HOST_STAGING=1 in the environment,
 * they are copied to the device first. */
int lbm_init_fields(LbmHandle* h, const void* phi, const void* u, int src_dtype,
                    int on_device, void* stream);

/* Advance nsteps time steps.  Replaces AllenCahnSolver.step
 * (lbm/fe_ac_solver.py:380-639).  Asynchronous on `stream`; no host sync. */
int lbm_step(LbmHandle* h, int nsteps, void* stream);

/* As lbm_step, with CUDA events recorded on `stream` before each step, between
 * its two kernels (before the fused kernel) and after the last step; on return
 * (synchronised) kernel_ms3[0] holds the summed duration of the phi kernels
 * (zero for the fused kernel), kernel_ms3[1] that of the update (or fused)
 * kernels and kernel_ms3[2] the whole span.  For measurement; same results as
 * lbm_step. */
int lbm_step_profiled(LbmHandle* h, int nsteps, void* stream, float* kernel_ms3);

/* Step kernel selection.  (0, 0, 0), the default, selects the two-kernel
 * streaming step (k_phi: phi and its grid sum, one thread per node; k_update:
 * the rest of the step, reading the phi stencil from L2).  Other extents
 * select the fused tiled kernel (one launch per step, phi recomputed on a
 * one-node halo in shared memory) with those tile extents, 2..64 for x and y
 * and 2..256 for z (an extent given as 0 is chosen automatically).  Results do
 * not depend on the choice; speed does.  lbm_get_tile returns (0, 0, 0) for
 * the two-kernel step.  No reference counterpart (a GB300 launch parameter). */
int lbm_set_tile(LbmHandle* h, int tx, int ty, int tz);
int lbm_get_tile(LbmHandle* h, int* txyz3);

/* Storage layout of the state arrays.  paired = 0 (the default): one
 * element per node in node order, stepped one thread per node.  paired = 1
 * (3-D grids with an even nx in LBM_F32 or LBM_F16 only): nodes x and
 * x + nx/2 of the same (y, z) share one 8-byte (float) or 4-byte (half) word
 * of every population, u and phi array, and the step runs one thread per such
 * pair with packed two-node loads, stores and f32x2 arithmetic: fewer
 * instructions per node, but at 128 registers per thread half as many
 * threads per SM (slower on the 150x150x107 ridge case on GB300).  Both layouts compute the same
 * step; they may differ in the last float32 bits (the compiler contracts
 * multiply-adds differently in the two kernels).  Call before
 * lbm_init_fields (LBM_E_STATE afterwards); LBM_E_UNSUPPORTED for a paired
 * request the grid or precision cannot take.  lbm_get_layout reports the
 * handle's layout.  No reference counterpart (a GB300 memory layout). */
int lbm_set_layout(LbmHandle* h, int paired);
int lbm_get_layout(LbmHandle* h, int* paired);

/* Step autotuner: times `reps` launches of the next step on the handle's
 * current state (which it leaves unchanged) for each candidate and keeps the
 * fastest: the two-kernel step with each phi-kernel work size (4, 8, 12, 16,
 * 24 or 32 nodes per thread) and each update-kernel block (128 or 256
 * threads; 256 only in the gradient-of-mu modes, and the paired layout's
 * update kernel has its fixed block), and each candidate tile shape of the
 * fused kernel.  Synchronises `stream`; allocates a temporary copy of u.
 * Outputs (may be NULL): the chosen extents and its time per launch in ms;
 * lbm_get_launch gives the chosen work size and block.  No reference
 * counterpart. */
int lbm_autotune(LbmHandle* h, int reps, void* stream, int* best_txyz3, float* best_ms);

/* Launch shape of the two-kernel step: the phi kernel's nodes per thread
 * (1..64) and the linear-layout update kernel's threads per block (128 or
 * 256; 256 in the gradient-of-mu modes).  Results do not depend on it; speed
 * does.  lbm_get_launch reports the shape in use (either output may be NULL;
 * the paired layout's update block is fixed at 128).  No reference
 * counterpart. */
int lbm_set_launch(LbmHandle* h, int phi_nodes_per_thread, int update_block);
int lbm_get_launch(LbmHandle* h, int* phi_nodes_per_thread, int* update_block);

/* Write the fields the reference exposes after the last step (or after
 * init) into caller device buffers of the handle's compute type (float for
 * LBM_F32 and LBM_F16, double for LBM_F64).  `mask` selects
 * LBM_FIELD_* bits; unselected pointers may be NULL.  Mirrors the attributes
 * phi, rho, u, P, p, mu_phi of AllenCahnSolver (lbm/fe_ac_solver.py:97-116,
 * values as assigned in step()). */
int lbm_get_fields(LbmHandle* h, uint32_t mask, void* phi, void* rho, void* u,
                   void* P, void* p, void* mu, void* stream);

/* Current populations f, g (19N each, 9N on a 2-D grid; caller device buffers of the handle's
 * compute type) as the reference holds them between steps (AllenCahnSolver.f/.g,
 * lbm/fe_ac_solver.py:97-98). */
int lbm_get_populations(LbmHandle* h, void* f, void* g, void* stream);

/* Inject a droplet mid-run: centre (3 doubles, lattice units), radius,
 * interface width xi, impact velocity (3 doubles, NULL = zero); a 2-D grid
 * reads the first two components of each.  As the
 * reference: phi becomes max(phi, C) where the droplet profile
 * C = 0.5 + 0.5 tanh(2 (R - |x - centre|) / xi) exceeds 0.1 (its core), u
 * becomes (1 - C) u + C u_impact everywhere, f and g are reset to their
 * equilibria (with the last step's pressure P) at the core nodes, solid
 * nodes keep phi = 0 and u = 0, the phi-mass reference becomes the new sum of
 * phi, and the next step has no previous phi u.  Until the next step the
 * fields read as after init_fields (P = 0, p = rho cs^2, the init laplacian
 * in mu_phi), where the reference keeps its last P and mu_phi.  core_nodes
 * (may be NULL; if given the call synchronises `stream`): the number of core
 * nodes.  Replaces AllenCahnSolver.inject_droplet (lbm/fe_ac_solver.py:645-732). */
int lbm_inject_droplet(LbmHandle* h, const double* center3, double radius, double xi, const double* u_impact3,
                       int64_t* core_nodes, void* stream);

/* Geometry tables as computed by lbm_set_geometry, into host buffers (any may
 * be NULL): node class byte (N), is_boundary (N), wall_normal (3N float32, 2N on a 2-D grid),
 * wall_weight (N float32), near_wall mask (N), partial mask (N).  Mirrors
 * ConningtonLeeWetting.is_boundary / wall_normal / wall_weight /
 * near_wall_mask (lbm/fe_wetting.py:140,147,305-306) and
 * AllenCahnSolver._partial_mask (lbm/fe_ac_solver.py:210). */
int lbm_get_geometry(LbmHandle* h, uint8_t* node_class, uint8_t* is_boundary,
                     float* wall_normal, float* wall_weight, uint8_t* near_wall,
                     uint8_t* partial);

/* Host-only form of the geometry precompute of lbm_set_geometry: needs no GPU
 * and no handle.  Wetting is enabled when theta_eq != 90 and kappa > 0; the
 * top-surface test uses `precision`.  Outputs as in lbm_get_geometry (any may
 * be NULL).  Same reference code as lbm_set_geometry
 * (lbm/fe_ac_solver.py:193-237, lbm/fe_wetting.py:122-311). */
int lbm_geometry_host(int64_t nx, int64_t ny, int64_t nz, const uint8_t* solid, const void* fraction,
                      int fraction_dtype, double theta_eq, double kappa, int precision,
                      uint8_t* node_class, uint8_t* is_boundary, float* wall_normal,
                      float* wall_weight, uint8_t* near_wall, uint8_t* partial);

/* Scalars: phi_mass_init (the reference's phi_mass_init), last step's sum of
 * phi, last mass-correction factor, number of steps taken. */
int lbm_get_scalars(LbmHandle* h, double* phi_mass_init, double* last_sum_phi,
                    double* last_correction, int64_t* step_count);

/* Spread diagnostics of the current phi on the device: out[0] volume = sum of
 * phi with solid zeroed, out[1] C_max, out[2..4] Dx, Dy, Dz extents of the
 * phi > 0.5 fluid set, out[5] k = Dx/Dy, out[6] z centre of mass of that set,
 * out[7] its node count, out[8] 1 if phi has a NaN else 0.  Host output,
 * synchronises `stream`.  On a 2-D grid Dz = 0 (as the reference reports for
 * 2-D fields) and out[6] is the centre along y.  Replaces measure_spread_factor
 * (lbm/fe_measure.py:11-82) and the every-50-steps extent/z_com/NaN check of
 * scripts/run_thesis_sweep.py:182-216. */
int lbm_measure(LbmHandle* h, double* out9, void* stream);

/* Global reductions of the current fields on the device, in float64: sum of
 * phi (solid nodes zeroed), total momentum sum rho(phi) u with rho = phi rho_l
 * + (1 - phi) rho_g, the first and last x, y, z index of the phi > 0.5 set
 * (extents6 = xmin, xmax, ymin, ymax, zmin, zmax; all -1 when the set is
 * empty) and the maximum of phi.  On a 2-D grid the z momentum is 0 and the
 * z extents are 0 (-1 when empty).  Host outputs (any may be NULL); synchronises
 * `stream`.  The mass/momentum guard of a solve and the data behind
 * measure_spread_factor (lbm/fe_measure.py:11-82). */
int lbm_reduce(LbmHandle* h, double* sum_phi, double* mom3, int32_t* extents6, float* cmax, void* stream);

/* Maximum node count of lbm_measure_static (its indexing is 32-bit). */
#define LBM_MEASURE_STATIC_MAX_NODES (1LL << 30)

/* Spread diagnostics of a caller's phi field that allocate nothing: no
 * cudaMalloc, no cudaFree, no allocating library call.  For callers that
 * cannot allocate device memory: code that runs inside a memory pool owned by
 * another runtime, host code under a driver that forbids allocation after
 * start-up, or a monitoring hook that must not disturb the allocator of the
 * solve it observes.  The reduction's block partials and its completion
 * counter live in a static device array of the library (1024 blocks x 11
 * doubles, about 90 KB, plus one counter), which every GPU that loads the
 * library holds until the process exits.
 *
 * phi: device, nx*ny*nz elements of phi_dtype (LBM_DT_F32 or LBM_DT_F64);
 * solid: device, nx*ny*nz bytes, 1 = solid, 0 = fluid (a torch.bool tensor);
 * out9: device, 9 doubles, written as by lbm_measure (volume, C_max, Dx, Dy,
 * Dz, k, z centre, count, NaN flag).  Asynchronous on `stream`.  Grids of more
 * than LBM_MEASURE_STATIC_MAX_NODES nodes are rejected with LBM_E_ARG.  A 2-D
 * (nx, ny) field passed as the grid 1 x nx x ny gets its x and y extents in
 * out9[3] and out9[4] and its centre along y in out9[6] (the reference's
 * 2-D Dx, Dy; its Dz is 0).
 *
 * The first call on a device looks up the static array's device address.
 * Under the CUDA runtime's default lazy module loading that lookup may load
 * the library's module onto the device, and loading places the static array
 * in device memory: an allocation made by the driver on the first call.  A
 * caller that may not allocate after start-up therefore makes one call per
 * device during start-up (or runs with CUDA_MODULE_LOADING=EAGER); the same
 * first call must come before any stream capture.  Later calls allocate
 * nothing.  The address is cached per device ordinal and belongs to the
 * device's primary context (the one the CUDA runtime uses); a caller that
 * makes another context current through the driver API must not call this.
 * Every call shares the one array and leaves its contents behind: calls
 * that overlap on the GPU (two streams, or two host threads on one device)
 * race and must be serialised by the caller.  No counterpart in the
 * reference: an addition of this library. */
int lbm_measure_static(int64_t nx, int64_t ny, int64_t nz, const void* phi, int phi_dtype,
                       const uint8_t* solid, double* out9, void* stream);

/*
 * Checkpoints.  A state blob holds everything the next step and the field
 * read-outs depend on: the current populations (the library's own pull-form
 * encoding), u, both phi buffers, the mass-correction factors, phi_mass_init
 * and the last sum of phi, the step count, the status flags and the step
 * sequencing flags.  It does not hold the configuration or the geometry: a
 * blob is loaded into a handle created with the same parameters, grid and
 * precision whose geometry was set from the same solid mask and fraction
 * (checked through a hash of the node-class table).  A run resumed from a blob
 * gives bit-identical results to the run that wrote it.  No reference
 * counterpart (the reference has no state checkpoint; its sweep drivers save
 * phi/u/solid snapshots, scripts/run_thesis_sweep.py:219-243).
 */
/* Size in bytes of the handle's state blob. */
int lbm_state_bytes(LbmHandle* h, int64_t* bytes);

/* Copy the state into a host buffer of exactly lbm_state_bytes bytes;
 * synchronises `stream`. */
int lbm_save_state(LbmHandle* h, void* host, int64_t bytes, void* stream);

/* Restore a state written by lbm_save_state (LBM_E_ARG if it belongs to another
 * grid, precision or geometry, or is not a state blob); synchronises `stream`. */
int lbm_load_state(LbmHandle* h, const void* host, int64_t bytes, void* stream);

/* Sticky status flags (LBM_STATUS_*) accumulated by the device; synchronises. */
int lbm_status(LbmHandle* h, uint32_t* flags);

/* Bytes of device memory lbm_create allocates for an nx*ny*nz grid of the
 * given precision (the admission size of a case).  The gradient-of-mu modes
 * (Cahn-Hilliard, mu_drive) add 4 arrays of the padded node count in the
 * compute type, a per-node amplification field one of N elements.  No GPU
 * needed.  No reference counterpart. */
int lbm_footprint(int64_t nx, int64_t ny, int64_t nz, int precision, int64_t* bytes);

/*
 * Batches: many independent grids (handles) that advance together, one launch
 * of each step kernel per time step for all of them (a block finds its case
 * in a block -> case table), replayed from a captured two-step CUDA graph.
 * Each case's arithmetic and reductions are its own, so its results are
 * bit-identical to stepping it alone.  The handles stay usable on their own
 * (fields, measure, ...) between batch calls and must outlive the batch.  No
 * reference counterpart: the reference steps one grid at a time (its sweep
 * drivers, scripts/run_thesis_sweep.py, loop over cases).
 */
typedef struct LbmBatch LbmBatch;

/* Batch of n handles of one precision on the current device, each with its
 * geometry set.  Allocates the case tables. */
int lbm_batch_create(LbmHandle* const* handles, int n, LbmBatch** out);

/* Advance every case by nsteps steps on `stream` (asynchronous).  If a case
 * is in its first step after init, every case takes that one step through the
 * single-grid kernels first.  Waits for the previous call's table upload. */
int lbm_batch_step(LbmBatch* b, int nsteps, void* stream);

/* Number of cases. */
int lbm_batch_size(LbmBatch* b, int* ncases);

/* Autotuner of the batched step's launch shape: the phi kernel's nodes per
 * thread (1, 2, 4, 8, 12, 16, 24 or 32: its block count per case) and the
 * update kernel's threads per block (128 or 256).  Times `reps` batched
 * steps that re-read the current state for each candidate pair and keeps the
 * fastest; the state is left unchanged.  Every case must have taken a step.
 * Synchronises `stream`; allocates temporary copies of u.  Outputs (may be
 * NULL): the chosen nodes per thread and the time per step in ms;
 * lbm_batch_get_launch gives both choices. */
int lbm_batch_autotune(LbmBatch* b, int reps, void* stream, int* best_per_thread, float* best_ms);

/* The batch's launch shape: phi-kernel nodes per thread and update-kernel
 * threads per block (either output may be NULL). */
int lbm_batch_get_launch(LbmBatch* b, int* phi_nodes_per_thread, int* update_block);

/* on = 1: every batched step is ONE cooperative launch (a grid of resident
 * blocks runs the phi work of every case, a grid-wide barrier, then the update
 * work of every case) instead of the two launches of the phi and update
 * kernels; on = 0 (the default): the two launches.  Same results bit for bit.
 * Linear-layout cases only (LBM_E_UNSUPPORTED otherwise); the update work
 * then runs 256-thread blocks.  No reference counterpart. */
int lbm_batch_set_cooperative(LbmBatch* b, int on);

/* Free the batch (not its handles). */
int lbm_batch_destroy(LbmBatch* b);

/* Legacy-VTK ASCII output of one snapshot, byte for byte the file of the
 * reference's write_vtk (io_utils/vtk_writer.py:10-86): `header` (the text up
 * to and including the POINT_DATA line, formatted by the caller), then the
 * density scalars, the velocity vectors and, if `solid` is not NULL, the solid
 * flags, each "%.6e" (NaN printed "nan") in the order of the caller's arrays
 * (npoints host values each; the reference writes C order, z fastest).  Host
 * only, no GPU needed.  Returns LBM_E_ARG if the file cannot be written. */
int lbm_write_vtk(const char* path, const char* header, int64_t npoints, const double* rho,
                  const double* ux, const double* uy, const double* uz, const int32_t* solid);

/* Message for the last error on the calling thread ("" if none). */
const char* lbm_last_error(void);

/* Library version string. */
const char* lbm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
