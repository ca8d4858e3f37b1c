/*
 * lbm.h -- C ABI of the GB300-native D2Q9 lattice-Boltzmann library (liblbm.so).
 *
 * This is the drop-in boundary for simuverse's fluid path.  Each entry point names the
 * reference interface it replaces (paths inside the simuverse project):
 *
 *   lbm_create            FluidSimulator::new      simuverse/src/fluid/fluid_simulator.rs:26-133
 *                         D2Q9Node::new            simuverse/src/fluid/d2q9_node.rs:31-209
 *   lbm_step              D2Q9Node::compute_by_pass simuverse/src/fluid/d2q9_node.rs:302-312
 *   lbm_compute           Simulator::compute       simuverse/src/fluid/fluid_simulator.rs:217-232
 *   lbm_reset             Simulator::reset         simuverse/src/fluid/fluid_simulator.rs:210-215
 *                         D2Q9Node::reset_lattice_info simuverse/src/fluid/d2q9_node.rs:247-261
 *   lbm_set_tau /
 *   lbm_update_viscosity  Simulator::update_uniforms simuverse/src/fluid/fluid_simulator.rs:175-193
 *   lbm_on_click          Simulator::on_click      simuverse/src/fluid/fluid_simulator.rs:137-152
 *   lbm_add_obstacle      D2Q9Node::add_obstacle   simuverse/src/fluid/d2q9_node.rs:215-245
 *   lbm_touch_begin       Simulator::touch_begin   simuverse/src/fluid/fluid_simulator.rs:154-156
 *   lbm_touch_move        Simulator::touch_move    simuverse/src/fluid/fluid_simulator.rs:158-173
 *   lbm_add_external_force D2Q9Node::add_external_force simuverse/src/fluid/d2q9_node.rs:263-300
 *   lbm_read_macro /
 *   lbm_read_macro_rgba16f the macro_tex the step writes  assets/wgsl/lbm/collide_stream.wgsl:36,74
 *   lbm_set_info/get_info the info buffer            simuverse/src/fluid/lattice.rs:5-24
 *
 * The remaining entry points (populations, conservation sums, checkpoints, the batched
 * form, the learned closure) have no counterpart in the reference; each says so.
 *
 * Conventions.  Every function returns an int status (LBM_OK = 0, negative on error,
 * LBM_IGNORED = 1 when the reference would silently ignore the request) and never
 * aborts; lbm_last_error() gives the message of the calling thread's last failure.
 * Host arrays are plain pointers owned by the caller.  Work is queued on the handle's
 * CUDA stream and the read functions synchronise that stream.  One handle must not be
 * used from two threads at once.
 *
 * Layout.  Cell (x, y) is x + y*nx with y growing downwards (screen rows, as in the
 * reference).  Populations are structure-of-arrays: direction i of cell c at c + i*N,
 * N = nx*ny (assets/wgsl/lbm/d2q9_fn.wgsl:13-17).  Direction order, vectors and
 * inverses follow simuverse/src/fluid/mod.rs:39-52:
 *   0:(0,0) 1:(1,0) 2:(0,-1) 3:(-1,0) 4:(0,1) 5:(1,-1) 6:(-1,-1) 7:(-1,1) 8:(1,1)
 */
#ifndef SIMUVERSE_GB300_LBM_H
#define SIMUVERSE_GB300_LBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_ABI_VERSION 1

/* status codes */
#define LBM_OK 0
#define LBM_IGNORED 1
#define LBM_ERR_ARG (-1)
#define LBM_ERR_CUDA (-2)
#define LBM_ERR_TIMEOUT (-3)
#define LBM_ERR_NAN (-4)
#define LBM_ERR_IO (-5)
#define LBM_ERR_STATE (-6)
#define LBM_ERR_NOMEM (-7)

/* step rules */
#define LBM_MODE_REFERENCE 0 /* the reference's shaders exactly: truncated weights, clamps,
                                forcing rows, wall-cell storage bounce-back */
#define LBM_MODE_PHYSICS 1   /* exact weights, no clamps, half-way bounce-back with moving
                                walls, Zou-He west inlet, zero-gradient east outflow */

/* population storage */
#define LBM_DTYPE_F32 0  /* reference mode: absolute f_i; physics mode: f_i - w_i */
#define LBM_DTYPE_F64 1  /* physics mode only: f_i - w_i in FP64, FP64 arithmetic */
#define LBM_DTYPE_F16 2  /* physics mode only: (f_i - w_i) * 2^10 in FP16, FP32 arithmetic */
#define LBM_DTYPE_BF16 3 /* physics mode only: f_i - w_i in BF16, FP32 arithmetic */

/* step kernel variants (physics mode) */
#define LBM_KERNEL_AUTO 0   /* the fastest measured variant: LBM_KERNEL_CELL for FP32 / FP64;
                               for FP16 / BF16 LBM_KERNEL_TILED where it applies, else
                               LBM_KERNEL_VEC2 (nx even) */
#define LBM_KERNEL_CELL 1   /* one cell per thread */
#define LBM_KERNEL_VEC4 2   /* four cells per thread, vector loads and stores (nx % 4 == 0) */
#define LBM_KERNEL_BULK 3   /* four cells per thread fed by double-buffered bulk asynchronous
                               copies into shared memory, persistent blocks (nx % 8 == 0) */
#define LBM_KERNEL_VEC2 4   /* two cells per thread, one 32-bit access per plane for 16-bit
                               storage (nx % 2 == 0) */
#define LBM_KERNEL_TILED 5  /* two cells per thread over a tiled layout of 16-bit populations
                               (the nine planes of 64 cells stored together; FP16 / BF16, BGK,
                               nx % 64 == 0); read-back and checkpoints are layout-independent
                               except that a checkpoint loads only into the same layout */
#define LBM_KERNEL_RING 6   /* the tiled layout and rules of LBM_KERNEL_TILED (same results bit
                               for bit), its rows staged in shared memory by bulk asynchronous
                               copies: blocks walk down strips of 8 tiles with a ring of rows
                               (slower than LBM_KERNEL_TILED on GB300) */

/* physics-mode collision */
#define LBM_COLLISION_BGK 0          /* single relaxation time */
#define LBM_COLLISION_REGULARIZED 1  /* BGK after projecting f_neq on the second-order Hermite
                                        moments (same viscosity) */
#define LBM_COLLISION_MRT 2          /* multiple relaxation times (Lallemand & Luo 2000 moments):
                                        stresses at 1/tau, energy 1.1, energy square 1.0, energy
                                        flux 1.2 */
#define LBM_COLLISION_KBC 3          /* entropic KBC: shear part at 1/tau (BGK's viscosity), higher
                                        moments at a per-cell entropic rate; stable for under-
                                        resolved turbulence near tau = 1/2 */

/* physics mode, FP16 / BF16 storage: rounding of the stored populations */
#define LBM_ROUNDING_NEAREST 0     /* round to nearest even */
#define LBM_ROUNDING_STOCHASTIC 1  /* stochastic rounding: a value between two stored neighbours is
                                      stored as the upper one with probability equal to its
                                      fractional position, so rounding errors have zero mean and
                                      slow gradients below the 16-bit spacing are kept on average;
                                      random bits from a hash of cell, step counter and seed
                                      (reproducible).  Runs on LBM_KERNEL_TILED, _VEC2 and
                                      _CELL (AUTO picks as for round-to-nearest). */

/* reference mode: floating-point evaluation of the shader rules (collide_stream.wgsl:40-87).
   Both keep every rule of the reference -- truncated weights and clamp maxima (mod.rs:39-49),
   the rho clamp (:49), the forcing rows' velocity replacement (:55-71), the population clamp
   (:79-83), the wall-cell storage of boundary.wgsl:28-31 -- and differ only in rounding. */
#define LBM_ARITH_EXACT 0 /* every WGSL operation rounded on its own (no multiply-add
                             contraction, IEEE divisions): bit-identical to the oracle */
#define LBM_ARITH_FAST 1  /* multiply-adds contracted, one reciprocal of rho, the
                             equilibrium evaluated on opposite pairs: within 1e-5 relative
                             of the exact form after one step, memory-bound speed */

/* initial masks */
#define LBM_SCENE_POISEUILLE 0 /* lattice.rs:62-83 (the only scene the reference UI builds) */
#define LBM_SCENE_CAVITY 1     /* lattice.rs:52-61 (reference); moving-lid box (physics) */
#define LBM_SCENE_CUSTOM 2     /* lattice.rs:47-51: box walls */
#define LBM_SCENE_CHANNEL 3    /* physics: walls y=0 and y=ny-1, parabolic Zou-He inlet at
                                  x=0, outflow at x=nx-1, seeded non-overlapping disks */
#define LBM_SCENE_PERIODIC 4   /* physics: no walls, periodic on both axes */

/* materials: lattice.rs:15-24 */
#define LBM_BULK 1
#define LBM_BOUNDARY 2
#define LBM_INLET 3
#define LBM_OBSTACLE 4
#define LBM_OUTLET 5
#define LBM_EXTERNAL_FORCE 6
#define LBM_GHOST 7

/* per-cell record, byte-compatible with LatticeInfo (lattice.rs:5-13) */
typedef struct lbm_lattice_info {
    int32_t material;
    int32_t block_iter; /* forcing countdown; -1 = permanent */
    float vx;           /* forcing / wall / inlet velocity */
    float vy;
} lbm_lattice_info;

typedef struct lbm_params {
    int32_t nx, ny;          /* lattice size (D2Q9Node::new derives it from the canvas) */
    int32_t mode;            /* LBM_MODE_* */
    int32_t dtype;           /* LBM_DTYPE_* */
    int32_t scene;           /* LBM_SCENE_* */
    float tau;               /* relaxation time; omega = 1/tau (mod.rs:32-36) */
    float lid_speed;         /* cavity lid velocity; reference literal 0.13 (lattice.rs:58) */
    float inlet_speed;       /* Poiseuille forcing 0.12 (lattice.rs:69); channel peak inlet u */
    float solid_fraction;    /* channel: solid fraction of the seeded disks */
    float disk_rmin, disk_rmax; /* channel: disk radius range (cells) */
    uint64_t seed;           /* channel: disk placement seed (mt19937_64) */
    int32_t pixel_size;      /* canvas pixels per lattice cell for on_click/touch_move */
    int32_t macro_every_step;/* 1: write the macro field every step, as the reference does;
                                0: only on the last step of each lbm_step call */
    int32_t kernel;          /* LBM_KERNEL_*: step kernel variant (results agree to rounding) */
    int32_t collision;       /* physics mode: LBM_COLLISION_* */
    int32_t rounding;        /* LBM_ROUNDING_* (16-bit storage; NEAREST otherwise) */
    int32_t arith;           /* reference mode: LBM_ARITH_* (physics mode ignores it) */
    int32_t reserved[2];
} lbm_params;

typedef struct lbm_handle lbm_handle;

/* library */
int lbm_abi_version(void);
const char* lbm_last_error(void);
void lbm_params_default(lbm_params* p);

/* lifetime -- FluidSimulator::new / drop.  lbm_destroy waits for the lattice's stream; work
   the caller queued on other streams that reads the lattice's buffers (lbm_device_populations,
   lbm_device_macro) must be complete before it is called. */
int lbm_create(const lbm_params* p, lbm_handle** out);
int lbm_destroy(lbm_handle* h);

/* Device memory of lattices.  lbm_create takes a lattice's buffers from a stream-ordered
   memory pool of the current device that the library owns, and lbm_destroy returns them there.
   The pool keeps up to `bytes` of returned memory reserved (default: an eighth of the device's
   memory, at most 16 GiB), so a lattice created after another was destroyed is served without
   a new device allocation.  lbm_memory_set_retain sets that limit for every device (0: give
   memory back at each synchronisation); lbm_memory_trim waits for the current device and gives
   its pool's unused memory back; lbm_memory_stats reads the current device pool's reserved and
   used bytes (0 and 0 before its first lattice).  Like every cached device state of the
   library, the pools belong to the device's primary context: a cudaDeviceReset invalidates
   them.  No counterpart in the reference (wgpu owns its buffers). */
int lbm_memory_set_retain(uint64_t bytes);
int lbm_memory_trim(void);
int lbm_memory_stats(uint64_t* reserved, uint64_t* used);
/* run the handle's work on a caller-owned cudaStream_t (NULL restores its own stream);
   no counterpart in the reference */
int lbm_set_stream(lbm_handle* h, void* cuda_stream);
int lbm_get_size(const lbm_handle* h, int32_t* nx, int32_t* ny);
int lbm_get_params(const lbm_handle* h, lbm_params* out);

/* stepping -- D2Q9Node::compute_by_pass (one call = collide+stream+boundary) */
int lbm_step(lbm_handle* h, int32_t nsteps);
/* Simulator::compute: one frame = two steps (swap 0 then 1) */
int lbm_compute(lbm_handle* h);
/* Simulator::reset / D2Q9Node::reset_lattice_info */
int lbm_reset(lbm_handle* h);
/* Simulator::update_uniforms: tau = 3*viscosity + 0.5 */
int lbm_update_viscosity(lbm_handle* h, float viscosity);
int lbm_set_tau(lbm_handle* h, float tau);

/* interaction -- Simulator::on_click / touch_begin / touch_move; canvas pixel coordinates */
int lbm_on_click(lbm_handle* h, float px, float py);
int lbm_add_obstacle(lbm_handle* h, int32_t x, int32_t y);
int lbm_touch_begin(lbm_handle* h);
int lbm_touch_move(lbm_handle* h, float px, float py);
int lbm_add_external_force(lbm_handle* h, float pos_x, float pos_y, float pre_x, float pre_y);

/* batched interaction on the GPU -- no single counterpart in the reference, which writes
   mask rows and records from the host one event at a time (d2q9_node.rs:215-300).  The
   list is applied in order with the result of the same sequence of single calls above
   (including the touch state), but the mask is written by two kernels on the handle's
   stream from a compact edit list and the call does not wait for the GPU.  applied (may be
   NULL) receives the number of edits that wrote the mask.  On an error nothing is applied. */
#define LBM_EDIT_OBSTACLE 0    /* a, b: lattice cell (lbm_add_obstacle) */
#define LBM_EDIT_CLICK 1       /* a, b: canvas pixel (lbm_on_click) */
#define LBM_EDIT_FORCE 2       /* a, b: position, c, d: previous position, canvas pixels
                                  (lbm_add_external_force) */
#define LBM_EDIT_TOUCH_BEGIN 3 /* lbm_touch_begin */
#define LBM_EDIT_TOUCH_MOVE 4  /* a, b: canvas pixel (lbm_touch_move) */
typedef struct lbm_edit {
    int32_t kind;
    float a, b, c, d;
} lbm_edit;
int lbm_apply_edits(lbm_handle* h, const lbm_edit* edits, int32_t n, int32_t* applied);

/* host-only mask helpers (no GPU needed; the handle functions above use the same code).
   lbm_build_mask: the scene mask of p (init_lattice_material, lattice.rs:26-98, for the
   reference scenes).  lbm_mask_add_obstacle: the disc of D2Q9Node::add_obstacle applied to a
   host array (rows y-28 .. y+27).  lbm_mask_force_stroke: the cells and record that
   D2Q9Node::add_external_force writes; it returns the number of cells written. */
int lbm_build_mask(const lbm_params* p, lbm_lattice_info* out);
/* the channel scene's disks (cx, cy, r per disk, FP64, cap disks at most) and their count in
   *n; physics-mode lattices build their scene mask on the device from this list, so it is all
   that lbm_create uploads for a channel.  No counterpart in the reference. */
int lbm_scene_disks(const lbm_params* p, double* out, int32_t cap, int32_t* n);
int lbm_mask_add_obstacle(int32_t nx, int32_t ny, lbm_lattice_info* info, int32_t x, int32_t y);
int lbm_mask_force_stroke(int32_t nx, int32_t ny, int32_t pixel_size, lbm_lattice_info* info, float pos_x,
                          float pos_y, float pre_x, float pre_y);

/* mask -- the info buffer (N records).  set_info replaces both the device buffer and the
   host copy that add_obstacle uploads rows from. */
int lbm_set_info(lbm_handle* h, const lbm_lattice_info* info);
int lbm_get_info(lbm_handle* h, lbm_lattice_info* out);

/* fields -- macro_tex (collide_stream.wgsl:36,74): rho (clamped in reference mode),
   ux, uy of the last step; walls give 0.  Any pointer may be NULL. */
int lbm_read_macro(lbm_handle* h, float* rho, float* ux, float* uy);
/* the rgba16float texel (ux, uy, rho, 1) / (0,0,0,0) on walls, as IEEE half bits */
int lbm_read_macro_rgba16f(lbm_handle* h, uint16_t* rgba);

/* populations -- no counterpart in the reference (its buffers are GPU-private).
   Absolute f_i as FP32 (dst_dtype LBM_DTYPE_F32) or FP64 (LBM_DTYPE_F64), 9*N values,
   the state the next step reads. */
int lbm_read_populations(lbm_handle* h, void* dst, int32_t dst_dtype);
int lbm_write_populations(lbm_handle* h, const void* src, int32_t src_dtype);
/* physics mode: equilibrium at (rho, ux, uy) host arrays of N floats (NULL: rho=1, u=0) */
int lbm_init_equilibrium(lbm_handle* h, const float* rho, const float* ux, const float* uy);

/* diagnostics -- no counterpart in the reference.  FP64 sums over non-solid cells of
   the absolute populations: out[0] mass, out[1] x momentum, out[2] y momentum;
   deterministic (fixed reduction order). */
int lbm_conservation(lbm_handle* h, double out[3]);
/* number of non-finite populations; returns LBM_ERR_NAN when it is not zero */
int lbm_check_finite(lbm_handle* h, uint64_t* count);
/* relative L2 errors of this handle's last macro field against ref's (same size):
   out[0] = |rho - rho_ref|_2 / |rho_ref|_2, out[1] = |u - u_ref|_2 / |u_ref|_2,
   out[2] = max |u - u_ref|, out[3] = max |rho - rho_ref| (FP64 sums over non-solid cells) */
int lbm_macro_error(lbm_handle* h, lbm_handle* ref, double out[4]);

/* checkpoint -- no counterpart in the reference.  Header (magic, version, nx, ny, mode,
   dtype, scene, tau, steps), then the raw state buffer, the info records and the host
   copy of the info records. */
int lbm_save(lbm_handle* h, const char* path);
int lbm_load(lbm_handle* h, const char* path);

/* Allocation-free FP64 sums -- no counterpart in the reference.  The same three sums as
   lbm_conservation (bit-identical for the same populations), computed over device
   buffers the caller owns: d_populations in the storage format of (mode, dtype) -- 9
   planes of nx*ny values, absolute f for reference mode, f - w (FP16: times 2^10) for
   physics mode; the tiled 16-bit layout of LBM_KERNEL_TILED / _RING is not accepted (its sums would
   be wrong without an error), so take such state from a handle with the SoA layout --
   d_info (device, nx*ny records; needed in physics mode to skip solids),
   d_out (device, 3 doubles).  For callers that cannot allocate device memory: a host
   application whose own runtime owns every device buffer, a process whose device memory
   is claimed by another allocator's pool, or a real-time loop that cannot afford
   cudaMalloc's device synchronisation.  The library allocates nothing on this path: its
   scratch is a fixed 29,184-byte array (1216 x 3 doubles) that every GPU loading the
   library keeps until exit.  Limit: lattices up to 2^30 cells (larger ones are rejected
   with LBM_ERR_ARG).  The first call on a device resolves the scratch address on that
   device (make it before any stream capture) and keeps it for the life of the process: it
   belongs to the device's primary context, the one the CUDA runtime uses, so the calls
   must run with that context current, and a cudaDeviceReset invalidates the kept address
   (do not call this entry point after one).  Calls share the scratch: calls that overlap
   on the GPU race.  Asynchronous on cuda_stream (NULL: the legacy default stream). */
int lbm_conservation_noalloc(const void* d_populations, int32_t dtype, int32_t mode, const lbm_lattice_info* d_info,
                             int32_t nx, int32_t ny, double* d_out, void* cuda_stream);

/* Bounds-checked builds -- no counterpart in the reference.  liblbm_bounds.so is this library
   compiled with LBM_BOUNDS_CHECK: the step kernels (reference mode, the one-cell physics step,
   the tiled 16-bit step, the bulk-copy step and the batched one-cell update) compare every
   population, flag and info index with the extent of its buffer before the access; an index
   outside it is counted with the first one's index, extent and access site, and the access is
   skipped (loads give 0), so nothing traps.  lbm_bounds_report returns the count since the
   last report on the current device (any pointer may be NULL) and clears it;
   lbm_bounds_selftest launches one thread that evaluates an index equal to its extent, with no
   memory access, so that the next report shows count 1 and site 99.  Both return
   LBM_ERR_STATE in the normal build. */
int lbm_bounds_report(uint64_t* count, uint64_t* first_index, uint64_t* first_limit, int32_t* first_site);
int lbm_bounds_selftest(void);

/* synchronises; LBM_ERR_TIMEOUT if a step kernel gave up on a bounded wait since creation
   -- no counterpart in the reference */
int lbm_status(lbm_handle* h);

/* counters -- no counterpart in the reference */
int lbm_steps_done(const lbm_handle* h, uint64_t* steps);
int lbm_kernel_launches(const lbm_handle* h, uint64_t* launches);

/* device views for in-GPU consumers (particles, colour mapping); valid until destroy.
   macro: 3 planes of N floats (rho, ux, uy).  No counterpart in the reference, whose
   consumers bind macro_tex directly. */
int lbm_device_macro(lbm_handle* h, float** rho, float** ux, float** uy);
/* the population buffer the next step reads, in the handle's storage format (see
   lbm_conservation_noalloc), valid until the next lbm_step, reset, load or destroy; *tiled
   (may be NULL) = 1 when it is in the tiled 16-bit layout of LBM_KERNEL_TILED / _RING, 0 for the
   plane-major SoA layout.  No counterpart in the reference. */
int lbm_device_populations(lbm_handle* h, void** d_state, int32_t* tiled);

/* ---------------------------------------------------------------------------------
   Consumers of the macro field, on the device (no texture or graphics interop).  Each
   reads the field the last lbm_step wrote, rounded to FP16 as the reference's
   rgba16float macro_tex holds it; before the first step the field is zero.
   --------------------------------------------------------------------------------- */

/* tracer particles -- the particle buffer and canvas of SettingObj (setting/setting_obj.rs)
   and the particle_update.wgsl dispatch FluidSimulator::compute runs after each step
   (fluid/fluid_simulator.rs:217-232) */
typedef struct lbm_particle_params {
    int32_t canvas_w, canvas_h; /* canvas pixels; canvas / pixel_size must give the lattice */
    int32_t count;              /* requested particles; the grid is lbm_particles_grid's */
    float life_time;            /* steps a particle lives before it restarts at its initial position */
    int32_t point_size;         /* side of the splatted square, pixels */
    float speed_factor;         /* pixels moved per lattice velocity unit (4.15 in the reference) */
    float fade_out_factor;      /* canvas alpha fade per present (0.96) */
    int32_t color_ty;           /* present colour: 0 direction hue, 1 speed hue, 2 uniform colour */
    float color[4];             /* uniform colour (color_ty 2) */
    uint64_t seed;              /* initial jitter (the reference draws from an unseeded generator) */
    int32_t deterministic;      /* 1: overlapping splats go to the highest particle index;
                                   0: plain racing stores, as the reference's dispatch */
    int32_t reserved[3];
} lbm_particle_params;

typedef struct lbm_particles lbm_particles;

void lbm_particle_params_default(lbm_particle_params* p);
/* get_particles_data (lib.rs:248-276): num_x = ceil(sqrt(count * w / h)), num_y = ceil(num_x * h / w) */
int lbm_particles_grid(int32_t canvas_w, int32_t canvas_h, int32_t count, int32_t* num_x, int32_t* num_y);
/* init_trajectory_particles (lib.rs:278-316) on the host: num_x * num_y records of 6 floats
   (pos x, pos y, initial x, initial y, life, fade), the reference's TrajectoryParticle;
   grid column x, row y is record x * num_y + y */
int lbm_particles_init_state(const lbm_particle_params* p, int32_t num_x, int32_t num_y, float* out);
int lbm_particles_create(lbm_handle* h, const lbm_particle_params* p, lbm_particles** out);
int lbm_particles_destroy(lbm_particles* ps);
int lbm_particles_info(const lbm_particles* ps, int32_t* num_x, int32_t* num_y);
/* one particle_update.wgsl pass over every particle, on h's stream */
int lbm_particles_update(lbm_particles* ps, lbm_handle* h);
/* present.wgsl (assets/wgsl/present.wgsl:15-54): RGBA (4 floats per pixel) of the canvas,
   then the alpha fade; *d_rgba (may be NULL) receives the device buffer */
int lbm_particles_present(lbm_particles* ps, lbm_handle* h, float** d_rgba);
int lbm_particles_read(lbm_particles* ps, float* out);
int lbm_particles_write(lbm_particles* ps, const float* in);
/* canvas: 3 floats per pixel (alpha, vx, vy), the reference's Pixel; rgba: the last present */
int lbm_particles_read_canvas(lbm_particles* ps, float* canvas, float* rgba);
int lbm_particles_counters(const lbm_particles* ps, uint64_t* updates, uint64_t* launches);

/* curl_update.wgsl:12-33: N floats, curl * 3.5 + 0.5 rounded to FP16, into a device buffer */
int lbm_curl(lbm_handle* h, float* d_out);

/* field colour maps, one RGBA (4 floats) per canvas pixel into a device buffer, the field
   sampled with linear filtering and clamp-to-edge addressing at each pixel centre */
#define LBM_COLOR_CURL 0  /* lbm/present.wgsl:18-40: hue curl, saturation 0.6 + 1.4 speed,
                             value 0.6 + 0.33 rho, alpha rho (d_curl from lbm_curl) */
#define LBM_COLOR_ANGLE 1 /* lbm/blend_img.wgsl:11-16: hue of atan2(ux, uy), opaque */
int lbm_colorize(lbm_handle* h, int32_t mode, const float* d_curl, int32_t canvas_w, int32_t canvas_h, float* d_rgba);

/* ---------------------------------------------------------------------------------
   Batched form -- no counterpart in the reference (simuverse runs one lattice).  Many
   independent physics-mode FP32 lattices (moving-lid cavities and channels) of uneven
   size advance together: in one cooperative persistent launch per lbm_batch_step call,
   replayed from a CUDA graph (LBM_BATCH_PERSISTENT), in one tile-list launch per step
   (LBM_BATCH_TILE_LAUNCHES), or in one launch per domain and step
   (LBM_BATCH_DOMAIN_LOOP).  The persistent kernel's grid barrier waits at most a set time;
   a timed-out wait sets an error that lbm_batch_status returns as LBM_ERR_TIMEOUT.
   --------------------------------------------------------------------------------- */
#define LBM_BATCH_PERSISTENT 0
#define LBM_BATCH_TILE_LAUNCHES 1
#define LBM_BATCH_DOMAIN_LOOP 2

typedef struct lbm_domain_desc {
    int32_t nx, ny;
    int32_t scene;  /* LBM_SCENE_CAVITY (lid at row 0 moving at speed) or LBM_SCENE_CHANNEL
                       (parabolic Zou-He inlet of peak speed, outflow, walls) */
    float tau;
    float speed;
    int32_t reserved[3];
} lbm_domain_desc;

typedef struct lbm_batch_config {
    int32_t tile_threads_x;   /* threads per tile row (multiple of 32) */
    int32_t tile_rows;        /* rows per tile (threads per block = tile_threads_x * tile_rows <= 256) */
    int32_t blocks_per_sm;    /* persistent grid = blocks_per_sm x SMs (0: occupancy maximum) */
    int32_t method;           /* LBM_BATCH_* */
    float ms_per_step;        /* filled by lbm_batch_tune */
    int32_t cells_per_thread; /* 1, or 4 (vector accesses); a tile is cells_per_thread * tile_threads_x wide */
    int32_t linear;           /* 1: a tile is a run of tile_threads_x * tile_rows consecutive cells of a
                                 domain's rows (no partly filled tiles at the right edge); needs
                                 cells_per_thread 1 and domains below 2^24 cells */
    int32_t full_occupancy;   /* one cell per thread: 1 = kernels compiled for 32 registers (8 blocks of
                                 256 threads per SM, some spills), 0 = for 40 (6 blocks) */
} lbm_batch_config;

typedef struct lbm_batch lbm_batch;

/* the seeded domain list: nx log-uniform in [64, 1024], ny = nx * aspect with aspect
   U[0.5, 2] (redrawn until ny is in [64, 1024]), tau U[0.55, 1], speed U[0.02, 0.1],
   cavity or channel with probability 1/2 (mt19937_64(seed)) */
int lbm_batch_generate(int32_t n, uint64_t seed, lbm_domain_desc* out);
int lbm_batch_create(int32_t n, const lbm_domain_desc* domains, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* b);
int lbm_batch_set_stream(lbm_batch* b, void* cuda_stream);
int lbm_batch_info(const lbm_batch* b, int32_t* ndomains, uint64_t* cells);
int lbm_batch_set_config(lbm_batch* b, const lbm_batch_config* cfg);
int lbm_batch_get_config(const lbm_batch* b, lbm_batch_config* cfg);
/* times trial_steps of every candidate tile shape and grid size, keeps the fastest
   (cached per shape class for the life of the process) */
int lbm_batch_tune(lbm_batch* b, int32_t trial_steps, lbm_batch_config* best);
int lbm_batch_step(lbm_batch* b, int32_t nsteps);
/* synchronises; LBM_ERR_TIMEOUT if a persistent launch's grid barrier timed out */
int lbm_batch_status(lbm_batch* b);
/* failure injection: a persistent launch in which `block` leaves before the barrier of
   `step`; the others time out after timeout_ns (0: the default 1 s).  Returns the status. */
int lbm_batch_inject_missing_arrival(lbm_batch* b, int32_t nsteps, int32_t block, int32_t step, uint64_t timeout_ns);
int lbm_batch_read_macro(lbm_batch* b, int32_t i, float* rho, float* ux, float* uy);
int lbm_batch_read_populations(lbm_batch* b, int32_t i, float* f);
int lbm_batch_read_info(lbm_batch* b, int32_t i, lbm_lattice_info* info);
int lbm_batch_conservation(lbm_batch* b, int32_t i, double out[3]);
int lbm_batch_counters(const lbm_batch* b, uint64_t* steps, uint64_t* launches);

/* ---------------------------------------------------------------------------------
   Learned closure of a coarsened lattice -- no counterpart in the reference.  A
   three-layer 3x3 convolution (9 -> 32 -> 32 -> 9 channels; BF16 weights and activations,
   FP32 accumulation on the tensor cores) maps 9 input channels of every coarse cell
   (lbm_closure_set_form) to a correction delta = P(y) / s_out of its populations; the
   projection P removes the density and momentum of the correction, per cell or as field
   means, so that the lattice's mass and momentum do not change.  Trained on the GPU (own forward,
   backward and Adam kernels) on pairs (coarse state C after k coarse steps from a
   coarse-grained fine state, coarse-grained fine state C* k * factor fine steps later),
   mean squared error against the target over the interior of square crops.  Closure lattices
   are physics-mode FP32 handles of the closure's size.
   --------------------------------------------------------------------------------- */
typedef struct lbm_closure lbm_closure;

/* number of logical parameters: W1[9][9][32], b1[32], W2[9][32][32], b2[32], W3[9][32][9],
   b3[9] ([tap][cin][cout]; tap 3 * (dy + 1) + (dx + 1) reads input cell (x + dx, y + dy)) */
int lbm_closure_param_count(void);
/* nx a multiple of 16; He-initialised from seed */
int lbm_closure_create(int32_t nx, int32_t ny, uint64_t seed, lbm_closure** out);
int lbm_closure_destroy(lbm_closure* c);
int lbm_closure_set_scales(lbm_closure* c, float s_in, float s_out);
/* the form of the closure (defaults: NEQ, POPULATIONS, CELL).  Inputs: s_in * f_neq of each
   cell, or s_in * (f_eq(rho, u) - w), which depends on the density and velocity fields only.
   Target of a pair (pred, target): s_out * (target - pred), s_out * (deq(rho*, u*) -
   deq(rho, u)), the difference of the equilibrium parts, or s_out * 3 w_i e_i . (j* - j),
   the momentum difference alone.  Projection: P cell by cell
   (no cell's density or momentum changes), or the field means of the output's density and
   momentum removed (the total mass and momentum of the lattice do not change, a cell's
   momentum may; a momentum target needs the field projection) */
#define LBM_CLOSURE_INPUT_NEQ 0
#define LBM_CLOSURE_INPUT_EQ 1
#define LBM_CLOSURE_TARGET_POPULATIONS 0
#define LBM_CLOSURE_TARGET_EQUILIBRIUM 1
#define LBM_CLOSURE_TARGET_MOMENTUM 2
/* the stress target (with the per-cell projection only): the correction is a momentum change
   in flux form, dj(x) = -1/2 sum_i e_i P(y)_i(x - e_i) / s_out, the lattice divergence of the
   projected outputs, added as 3 w_i e_i . dj -- no cell's density changes and the lattice's
   total momentum does not either (a divergence sums to zero): a learned sub-grid stress.  The
   loss compares its effect over the pair's window of n coarse steps with an application every k
   steps, -factor sum_i e_i P(y)_i(x - e_i) with factor = n / (2 k)
   (lbm_closure_set_stress_factor), with the momentum difference j(target) - j(pred). */
#define LBM_CLOSURE_TARGET_STRESS 3
#define LBM_CLOSURE_PROJECT_CELL 0
#define LBM_CLOSURE_PROJECT_DOMAIN 1
int lbm_closure_set_form(lbm_closure* c, int32_t inputs, int32_t target, int32_t projection);
/* the stress target's factor n / (2 k): window of a pair in coarse steps over twice the
   interval between applications (default 0.5: one application per step over one step) */
int lbm_closure_set_stress_factor(lbm_closure* c, float factor);
/* kernels of the closure.  FUSED (default): lbm_closure_apply / lbm_closure_predict compute the
   features and the three layers in one kernel on the tcgen05 tensor cores with the activations
   in shared and tensor memory, and training computes the weight gradients on the tcgen05 tensor
   cores (crops a multiple of 64 wide; others on the CUDA cores).  LAYERS: the feature kernel and
   one mma.sync kernel per layer with the activations in device memory, and the weight gradients
   on the CUDA cores.  Both give the same network within BF16 rounding of the activations, and
   the same gradients within FP32 summation order. */
#define LBM_CLOSURE_KERNEL_FUSED 0
#define LBM_CLOSURE_KERNEL_LAYERS 1
int lbm_closure_set_kernel(lbm_closure* c, int32_t kernel);
/* synchronises; LBM_ERR_TIMEOUT if the fused kernel gave up on a bounded wait since creation */
int lbm_closure_status(lbm_closure* c);
int lbm_closure_get_params(lbm_closure* c, float* out);
int lbm_closure_set_params(lbm_closure* c, const float* in);
/* coarse = block average over factor x factor cells of the fine lattice's density and
   momentum, equilibrium of those, plus neq_scale times the block-averaged f_neq */
int lbm_coarsen(lbm_handle* fine, lbm_handle* coarse, int32_t factor, float neq_scale);
/* adds the network's correction to h's current populations (periodic convolution),
   asynchronously on h's stream */
int lbm_closure_apply(lbm_closure* c, lbm_handle* h);
/* correction of the whole lattice without applying it: 9 planes of nx * ny floats */
int lbm_closure_predict(lbm_closure* c, lbm_handle* h, float* delta_out);
/* training storage: up to max_pairs pairs of crop x crop windows, batches of `batch` */
int lbm_closure_reserve(lbm_closure* c, int32_t max_pairs, int32_t crop, int32_t batch);
/* stores the crop at (ox, oy) (periodic) of the pair (pred, target) */
int lbm_closure_add_pair(lbm_closure* c, lbm_handle* pred, lbm_handle* target, int32_t ox, int32_t oy);
int lbm_closure_pairs(const lbm_closure* c, int32_t* n);
/* Adam on random batches; loss_out (may be NULL): mean loss of the last iteration */
int lbm_closure_train(lbm_closure* c, int32_t iters, float lr, uint64_t seed, double* loss_out);
/* mean loss over stored pairs [begin, end), parameters unchanged */
int lbm_closure_eval(lbm_closure* c, int32_t begin, int32_t end, double* loss_out);
/* forward + backward on host crops feats, targets ([nimg][size][size][9], feature and
   output units); grads: lbm_closure_param_count() floats */
int lbm_closure_loss_grad(lbm_closure* c, int32_t nimg, int32_t size, const float* feats, const float* targets,
                          double* loss_out, float* grads);
int lbm_closure_counters(const lbm_closure* c, uint64_t* launches, uint64_t* adam_steps);

#ifdef __cplusplus
}
#endif
#endif
