/*
 * lbm_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of simuverse's D2Q9 lattice-Boltzmann step, used only by tests/,
 * by __graft_entry__.smoke() to check results, and by bench.py's CPU-baseline leg.
 * The CUDA library (simuverse_gb300/csrc) never links or calls it.
 *
 * Parity status: UNPINNED. The reference is Rust + WGSL executed through wgpu; no Rust
 * toolchain and no graphics API exist on either machine, and the reference's own tests
 * hold no vectors for this path. The restatement is cross-checked against an independent
 * pure-Python restatement (oracle/pyref.py) and against analytic physics cases.
 *
 * Layout (same as the reference, d2q9_fn.wgsl:13-17): population of direction i at cell
 * (x, y) lives at index x + y*nx + i*N with N = nx*ny.  Direction order and vectors follow
 * simuverse/src/fluid/mod.rs:39-52 (y grows downwards, screen rows).
 */
#ifndef SIMUVERSE_GB300_LBM_ORACLE_H
#define SIMUVERSE_GB300_LBM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* simuverse/src/fluid/lattice.rs:5-13 (16 bytes, AoS) */
typedef struct {
    int32_t material;
    int32_t block_iter;
    float vx;
    float vy;
} lo_info;

/* ---------------- reference mode (restates the WGSL shaders) ---------------- */

/* lattice.rs:26-98; scene 0 Poiseuille, 1 lid-driven cavity, 2 custom box.
 * lid_vx / inlet_vx replace the literals 0.13 / 0.12 (lattice.rs:57-59, 68-70). */
void lo_mask_reference(int nx, int ny, int scene, float lid_vx, float inlet_vx, lo_info* info);

/* init.wgsl:19-63.  fluid_ty: 0 Poiseuille-style init, 1 plain w_i (d2q9_node.rs:53-57). */
void lo_ref_init(int nx, int ny, int fluid_ty, lo_info* info, float* A, float* B);

/* collide_stream.wgsl:25-88 followed by boundary.wgsl:3-35 (d2q9_node.rs:302-312).
 * A: collide_cell (read), B: stream_cell (written).  macro4 (N*4 floats, may be NULL)
 * receives (ux, uy, rho, w) per cell as stored to macro_tex.  scratch: 9*N floats.
 * The boundary pass is executed in a fixed two-phase order (read every moved value,
 * then write the moved values, then the zeros), which is one of the orders the
 * reference's racy GPU dispatch can produce. */
void lo_ref_step(int nx, int ny, float omega, lo_info* info, const float* A, float* B,
                 float* macro4, float* scratch);

/* d2q9_node.rs:215-245 (disc of radius 28 at lattice cell (x, y), rows y-28 .. y+27).
 * host_info is the host-side copy (D2Q9Node::lattice_info_data); rows [y-28, y+28)
 * of it are copied into dev_info, exactly as the reference uploads them. Returns 0, or
 * -1 if the rows fall outside the lattice (the reference would index out of range). */
int lo_add_obstacle(int nx, int ny, lo_info* host_info, lo_info* dev_info, int x, int y);

/* simuverse_app/fluid_simulator.rs:137-152 guard + the call above; canvas coordinates. */
int lo_on_click(int nx, int ny, int pixel_size, lo_info* host_info, lo_info* dev_info,
                float px, float py);

/* d2q9_node.rs:263-300: a force stroke from pre (canvas px) to pos (canvas px). */
void lo_add_external_force(int nx, int ny, int pixel_size, lo_info* dev_info,
                           float pos_x, float pos_y, float pre_x, float pre_y);

/* ---------------- physics mode (exact weights, no clamps) ---------------- */
/* Storage is the shifted deviation d_i = f_i - w_i.
 * Materials: 1,7 fluid; 2,4 solid (half-way bounce-back; a solid with (vx,vy) != 0 is a
 * moving wall); 3 Zou-He velocity inlet on a west face with (vx,vy); 5 zero-gradient
 * outflow on an east face; 6 Guo body force (vx,vy) with the reference's block_iter
 * countdown.  Periodic wrap on both axes where no boundary intervenes. */
void lo_phys_step_f32(int nx, int ny, float omega, lo_info* info, const float* A, float* B,
                      float* macro3 /* rho, ux, uy planes; may be NULL */, int collision /* 0 BGK, 1 regularised */);
void lo_phys_step_f64(int nx, int ny, double omega, lo_info* info, const double* A, double* B,
                      double* macro3, int collision);
/* equilibrium initialisation from macro fields (NULL -> rho=1, u=0); solids get 0 */
void lo_phys_init_f32(int nx, int ny, const lo_info* info, const float* rho, const float* ux,
                      const float* uy, float* A);
void lo_phys_init_f64(int nx, int ny, const lo_info* info, const double* rho, const double* ux,
                      const double* uy, double* A);

/* physics masks: 1 cavity (moving lid on row y=0), 3 channel, 4 periodic */
void lo_mask_physics_cavity(int nx, int ny, float lid_vx, lo_info* info);
/* channel with Zou-He parabolic inlet (peak u_max), outflow, walls y=0, y=ny-1 and
 * seeded non-overlapping disks (mt19937_64); returns the number of disks placed */
int lo_mask_physics_channel(int nx, int ny, float u_max, uint64_t seed, float solid_fraction,
                            float rmin, float rmax, lo_info* info);

/* FP64 sums over non-solid cells of the absolute populations: out = {mass, jx, jy} */
void lo_conservation_dev_f32(int nx, int ny, const lo_info* info, const float* A, double out[3]);
void lo_conservation_dev_f64(int nx, int ny, const lo_info* info, const double* A, double out[3]);

/* ---------------- consumers of the macro field (lbm_oracle_view.inc) ---------------- */
float lo_h16(float v); /* nearest FP16 value, ties to even */
void lo_particles_grid(int cw, int ch, int count, int* num_x, int* num_y);
/* records of 6 floats: pos x, pos y, initial x, initial y, life, fade */
void lo_particles_init(int cw, int ch, int num_x, int num_y, float life_time, uint64_t seed, float* out);
/* ux, uy: the FP32 macro planes (rounded to FP16 inside); zero: no step since init */
void lo_particles_update(int nx, int ny, const float* ux, const float* uy, int zero, float lattice_pixel,
                         float life_time, float speed_factor, int point_size, int cw, int ch, int poiseuille,
                         int count, float* state, float* canvas);
void lo_present_canvas(int npix, int color_ty, int speed_ty, float fade_out, const float* rgb, float* canvas,
                       float* rgba);
void lo_curl(int nx, int ny, const float* ux, const float* uy, int zero, float* out);
void lo_colorize(int nx, int ny, const float* rho16, const float* ux16, const float* uy16, const float* curl, int cw,
                 int ch, int mode, float* rgba);

/* number of OpenMP threads the oracle uses */
int lo_num_threads(void);
void lo_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
