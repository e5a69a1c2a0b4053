/*
 * eqfluid.h -- C ABI of the GB300-native (sm_103a) stable-fluids frame step.
 *
 * This is the drop-in boundary for Equilibrium's solver
 * (vkabadzhova/equilibrium, src/simulation/fluid.rs). A Rust (or any other)
 * host binds these functions with a plain `extern "C"` block; no C++ or torch
 * type crosses the boundary: only opaque handles, plain pointers, sizes and
 * IEEE-754 scalars.
 *
 * State layout. A handle owns the six f32 arrays of `Fluid` (fluid.rs:59-77),
 * each `size * size` cells including the ghost frame, x fastest
 * (idx = x + y*size, fluid.rs:31-35), plus the wall mask `cells_type`
 * (fluid.rs:80) as one byte per cell: 1 = DefaultWall, 0 = NoWall. Host
 * buffers passed to the read/write functions use exactly that dense layout.
 * On the device the rows are padded to a 128-byte pitch.
 *
 * Errors. Every function returns EQ_OK (0) or a positive EQ_ERR_* code; the
 * reference panics in the same places (Rectangle::new, obstacle.rs:67),
 * which a Rust wrapper reproduces by panicking on a non-zero return.
 * eq_last_error() gives a message for the calling thread's last failure.
 *
 * Threading. One handle is used by one host thread at a time (the reference
 * moves a Fluid into its simulation thread and clones it per frame,
 * renderer.rs:125-128, renderer_helpers.rs:61-64). Each handle owns a CUDA
 * stream on its device; every entry point selects that device first, so a
 * handle may be driven from any host thread.
 *
 * Arithmetic. The plain step is bit-identical to the reference's f32 step:
 * kernels use explicitly rounded adds and multiplies (never contracted into
 * FMA), IEEE division, the reference's evaluation order and its quirks
 * (advect's row break, aliasing of the six arrays, obstacle-blind scalar
 * boundaries).
 */
#ifndef EQFLUID_H
#define EQFLUID_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EQ_ABI_VERSION 1

/* Status codes. */
#define EQ_OK 0
#define EQ_ERR_ARG 1     /* invalid argument (size, field, rectangle, mask frame) */
#define EQ_ERR_CUDA 2    /* a CUDA runtime call failed */
#define EQ_ERR_TIMEOUT 3 /* a bounded inter-block wait ran out (device error word) */
#define EQ_ERR_OOM 4     /* device or host allocation failed */
#define EQ_ERR_STATE 5   /* handle in an unusable state */

/* Field indices: the six arrays of Fluid in declaration order (fluid.rs:59-77). */
#define EQ_FIELD_SCRATCH 0 /* scratch_space (private in the reference) */
#define EQ_FIELD_DENSITY 1 /* pub density */
#define EQ_FIELD_VX 2      /* pub velocities_x */
#define EQ_FIELD_VY 3      /* pub velocities_y */
#define EQ_FIELD_VX0 4     /* velocities_x0 (private) */
#define EQ_FIELD_VY0 5     /* velocities_y0 (private) */

/* Orientation (fluid.rs:21-29). */
#define EQ_MODE_ADJUST_ROW 0
#define EQ_MODE_ADJUST_COLUMN 1
#define EQ_MODE_PASSIVE 2

/* SimulationConfigs (configs.rs:5-12). `frames` is both the app's frame count
 * and the Gauss-Seidel sweep count of every lin_solve (fluid.rs:312). */
typedef struct eq_simulation_configs {
  float delta_t;
  int64_t frames;
  uint32_t size; /* cells per side including the ghost frame */
} eq_simulation_configs;

/* FluidConfigs (configs.rs:37-48); the two display colours stay on the host. */
typedef struct eq_fluid_configs {
  float diffusion;
  float viscousity;
  int32_t has_perlin_noise;
} eq_fluid_configs;

typedef struct eq_fluid eq_fluid; /* opaque; owns device state */

/* ---- lifecycle --------------------------------------------------------- */

/* Fluid::new (fluid.rs:93-110): zeroed arrays, all NoWall, then init()
 * (fluid.rs:602-606): vx = vy = 1 everywhere, +0.9 density (and scratch) on
 * the 21x21 block centred at size/2, frame = DefaultWall. Requires
 * size >= 20 (smaller sizes underflow `size/2 - 10`, fluid.rs:534) and
 * frames >= 0. `device` < 0 means the current CUDA device. */
int eq_fluid_new(const eq_fluid_configs* fluid, const eq_simulation_configs* sim,
                 int device, eq_fluid** out);

/* Fluid::default (fluid.rs:83-89): new() with the default configs
 * (configs.rs:14-22, 50-60), then init() a second time (velocities 2.0,
 * block density 1.8). */
int eq_fluid_default(int device, eq_fluid** out);

/* Re-applies init() (fluid.rs:602-606) on top of the current state. */
int eq_fluid_init(eq_fluid* h);

/* #[derive(Clone)] (fluid.rs:51): a deep device-to-device copy. */
int eq_fluid_clone(const eq_fluid* h, eq_fluid** out);

/* Drop: frees the device state. Accepts NULL. */
int eq_fluid_free(eq_fluid* h);

int eq_fluid_get_configs(const eq_fluid* h, eq_fluid_configs* fluid,
                         eq_simulation_configs* sim);

/* Changes delta_t / frames / diffusion / viscousity (the pub config fields,
 * fluid.rs:54-56). `size` must stay the same. */
int eq_fluid_set_configs(eq_fluid* h, const eq_fluid_configs* fluid,
                         const eq_simulation_configs* sim);

/* ---- the hot path ------------------------------------------------------ */

/* Fluid::step (fluid.rs:437-524): diffuse vx/vy, project, advect vx/vy,
 * project, diffuse + advect density, scratch = density. Asynchronous on the
 * handle's stream; returns after launching. */
int eq_fluid_step(eq_fluid* h);

/* `nframes` consecutive steps. */
int eq_fluid_step_n(eq_fluid* h, int64_t nframes);

/* Blocks until the handle's stream is idle and reports any device-side
 * error (EQ_ERR_TIMEOUT when a bounded wait ran out). */
int eq_fluid_synchronize(eq_fluid* h);

/* ---- sources (fluid.rs:120-131) ---------------------------------------- */

/* add_density: density[idx] += amount; scratch[idx] += amount, with idx!'s
 * clamping of (x, y) into the grid (fluid.rs:31-35). */
int eq_fluid_add_density(eq_fluid* h, uint32_t x, uint32_t y, float amount);

/* add_velocity: vx[idx] += amount_x; vy[idx] += amount_y. */
int eq_fluid_add_velocity(eq_fluid* h, uint32_t x, uint32_t y, float amount_x,
                          float amount_y);

/* n sources from HOST arrays, applied in array order: for each s,
 * add_density(x[s], y[s], density[s]) and add_velocity(x[s], y[s], vx[s],
 * vy[s]). Any of density/vx/vy may be NULL (treated as no contribution). */
int eq_fluid_add_sources(eq_fluid* h, int64_t n, const uint32_t* x, const uint32_t* y,
                         const float* density, const float* vx, const float* vy);

/* `nframes` frames, each = that frame's sources then step(), with the sources
 * read from DEVICE arrays of shape [nframes][nsrc] (frame-major). This is
 * the form a frame loop with pre-staged inputs uses. */
int eq_fluid_run_device_sources(eq_fluid* h, int64_t nframes, int64_t nsrc,
                                const uint32_t* d_x, const uint32_t* d_y,
                                const float* d_density, const float* d_vx,
                                const float* d_vy);

/* ---- obstacles (fluid.rs:610-619, obstacle.rs:55-87) ------------------ */

/* Rectangle::new validation: EQ_OK if dl.x < ur.x, dl.y < ur.y and all four
 * coordinates are < size, else EQ_ERR_ARG (the reference panics). */
int eq_rectangle_check(int64_t dl_x, int64_t dl_y, int64_t ur_x, int64_t ur_y,
                       uint32_t size);

/* fill_obstacle: marks [x0,x1) x [y0,y1) as DefaultWall (clamped idx!). */
int eq_fluid_fill_obstacle(eq_fluid* h, int64_t x0, int64_t y0, int64_t x1, int64_t y1);

/* ---- the pub fields: host <-> device ------------------------------------ */

/* Dense size*size copies. `n` is the element count of the host buffer and
 * must equal size*size. Reads synchronise the handle's stream. */
int eq_fluid_read_field(eq_fluid* h, int field, float* host, uint64_t n);
int eq_fluid_write_field(eq_fluid* h, int field, const float* host, uint64_t n);

/* Asynchronous variants on the handle's stream (host memory should be pinned
 * for true asynchrony); complete at the next eq_fluid_synchronize. */
int eq_fluid_read_field_async(eq_fluid* h, int field, float* host, uint64_t n);
int eq_fluid_write_field_async(eq_fluid* h, int field, const float* host, uint64_t n);

/* `count` (1..6) fields at once, field k into host[k] (n = size*size each):
 * one device-side packing and one contiguous copy per field, then one
 * synchronisation (the pub fields a frame loop reads back after each step:
 * density, velocities_x, velocities_y). */
int eq_fluid_read_fields(eq_fluid* h, int count, const int* fields, float* const* host,
                         uint64_t n);

/* The same without waiting: the fields are packed on the handle's stream
 * (the next step's kernels may follow at once) and copied to host[k] on a
 * read-back stream of their own, so a frame loop's read-back of frame n
 * overlaps the computation of frame n+1 (two staging buffers, used in turn).
 * host[k] must stay valid, and should be pinned, until the copy is complete:
 * at the next eq_fluid_synchronize, which waits for every read-back (and
 * reports a device error of the steps before). */
int eq_fluid_read_fields_async(eq_fluid* h, int count, const int* fields, float* const* host,
                               uint64_t n);

/* cells_type (fluid.rs:80) as bytes, 1 = DefaultWall. A written mask must keep
 * the whole ghost frame as DefaultWall (init_walls, fluid.rs:552-570, makes it
 * so and nothing in the reference clears it); otherwise EQ_ERR_ARG. */
int eq_fluid_read_cells(eq_fluid* h, uint8_t* host, uint64_t n);
int eq_fluid_write_cells(eq_fluid* h, const uint8_t* host, uint64_t n);

/* ---- around the step --------------------------------------------------- */

/* RGBA colours of render_image (renderer_helpers.rs:115-180): FluidConfigs'
 * fluid_color and world_color (configs.rs:37-60) and the listener's
 * obstacles_color. NULL selects the defaults (208,88,157,220), (94,146,162,128)
 * and red (255,0,0,255). */
typedef struct eq_render_colors {
  uint8_t fluid[4];
  uint8_t world[4];
  uint8_t obstacles[4];
} eq_render_colors;

/* The frame's image, size x size RGBA8 pixels (x fastest, pixel (x, y) =
 * cell idx(x, y)), by render_image's rule: a wall in the obstacles colour, a
 * fluid cell with density != 0 as ((density*fluid.r) as u8, fluid.g,
 * density as u8, 1) with Rust's saturating casts, any other cell in the world
 * colour. The host form synchronises; the device form writes a caller's
 * device buffer on the handle's stream (a headless frame buffer). */
int eq_fluid_render_rgba(eq_fluid* h, const eq_render_colors* colors, uint8_t* host_rgba,
                         uint64_t nbytes);
int eq_fluid_render_rgba_device(eq_fluid* h, const eq_render_colors* colors, void* d_rgba);

/* add_noise (fluid.rs:575-599) on the device: a velocity impulse at the
 * centre cell equal to twice the point (rx, ry) rotated about the centre by
 * eq_noise_angle(delta_t) degrees, (rx, ry) uniform over the grid from a
 * counter-based generator seeded by `seed` (the handle's noise counter
 * advances each call). The reference draws (rx, ry) from thread_rng and the
 * angle from the `noise` crate's Perlin, so results match it in distribution
 * only. */
int eq_fluid_add_noise(eq_fluid* h, uint64_t seed);
double eq_noise_angle(float delta_t); /* gradient noise at (dt, dt) * 6.28 * 2 */

/* fill_obstacle (fluid.rs:610-619) rasterised on the device: the device mask
 * and the boundary codes are updated in place (no host upload); the host copy
 * of cells_type is kept current. */
int eq_fluid_fill_obstacle_device(eq_fluid* h, int64_t x0, int64_t y0, int64_t x1, int64_t y1);

/* The frame loop of CurrentSimulation::simulate (renderer_helpers.rs:52-72)
 * without a host synchronisation per frame: `nframes` frames of (optional
 * device add_noise, then step) captured once into a CUDA graph (kept for the
 * next call with the same arguments and configs) and replayed. Asynchronous. */
int eq_fluid_step_graph(eq_fluid* h, int64_t nframes, int32_t with_noise, uint64_t seed);

/* ---- single phases (the reference's private functions), on fields ------- */

/* set_boundaries (fluid.rs:252-272) on one field. */
int eq_fluid_set_boundaries(eq_fluid* h, int mode, int field);

/* lin_solve (fluid.rs:301-325): `frames` Gauss-Seidel sweeps of
 * x = (x0 + a*(x[i+1]+x[i-1]+x[j+1]+x[j-1])) / c, each followed by
 * set_boundaries(mode). x_field != x0_field. */
int eq_fluid_lin_solve(eq_fluid* h, int mode, int x_field, int x0_field, float a, float c);

/* diffuse (fluid.rs:276-298): lin_solve with a = dt*diff*(size-2)^2, c = 1+4a. */
int eq_fluid_diffuse(eq_fluid* h, int mode, int x_field, int x0_field, float diffusion);

/* project (fluid.rs:330-375) on four distinct fields. */
int eq_fluid_project(eq_fluid* h, int vx_field, int vy_field, int p_field, int div_field);

/* advect (fluid.rs:378-432); d_field must differ from d0/u/v. */
int eq_fluid_advect(eq_fluid* h, int mode, int d_field, int d0_field, int u_field,
                    int v_field);

/* ---- batches of independent scenes -------------------------------------- */

/* Many independent Fluid states (fluid.rs:52-81), each with its own size,
 * delta_t, sweep count (`frames`), diffusion and viscousity, advanced
 * together: eq_batch_step runs Fluid::step (fluid.rs:437-524) once per frame
 * on every scene. The reference has one Fluid per simulation thread
 * (renderer.rs:125-128); a batch replaces N such threads. Every scene's result
 * is bit-identical to stepping an eq_fluid of the same configs (and to the
 * reference's f32 step): a scene is computed by one thread block with the
 * reference's operation order, and scenes never interact. */
typedef struct eq_scene_desc {
  uint32_t size; /* cells per side including the ghost frame, >= 20 */
  float delta_t;
  int64_t frames; /* Gauss-Seidel sweeps per lin_solve (fluid.rs:312) */
  float diffusion;
  float viscousity;
} eq_scene_desc;

typedef struct eq_batch eq_batch; /* opaque; owns device state */

/* Creates `nscenes` scenes, each in the Fluid::new state (fluid.rs:93-110:
 * init() once, frame = DefaultWall). `device` < 0 = current device. */
int eq_batch_new(int64_t nscenes, const eq_scene_desc* scenes, int device, eq_batch** out);
/* The same with the fields STORED in FP16 or BF16 (storage EQ_STORE_F16 /
 * EQ_STORE_BF16, defined with the precision form below; 0 = FP32), or with
 * only density and scratch in FP16 (EQ_STORE_F16_SCALARS): every phase
 * computes exactly as the FP32 batch on the widened values and rounds once on
 * store, so the per-scene results differ from the reference's only by those
 * roundings (and their propagation). */
int eq_batch_new_storage(int64_t nscenes, const eq_scene_desc* scenes, int storage, int device,
                         eq_batch** out);
int eq_batch_free(eq_batch* b); /* accepts NULL */
int eq_batch_scene_count(const eq_batch* b, int64_t* n);
/* Sum over scenes of (size-2)^2: the interior cells one frame advances. */
int eq_batch_cell_count(const eq_batch* b, uint64_t* interior_cells);

/* fill_obstacle (fluid.rs:610-619) on one scene: [x0,x1) x [y0,y1) walls. */
int eq_batch_fill_obstacle(eq_batch* b, int64_t scene, int64_t x0, int64_t y0, int64_t x1,
                           int64_t y1);
int eq_batch_read_cells(eq_batch* b, int64_t scene, uint8_t* host, uint64_t n);

/* Per-scene sources applied before every step, in array order:
 * add_density(x, y, density) then add_velocity(x, y, vx, vy) for each s
 * (fluid.rs:120-131). NULL value arrays count as zeros; n = 0 clears. */
int eq_batch_set_sources(eq_batch* b, int64_t scene, int64_t n, const uint32_t* x,
                         const uint32_t* y, const float* density, const float* vx,
                         const float* vy);

/* Dense size*size copies of one scene's field (synchronous). */
int eq_batch_read_field(eq_batch* b, int64_t scene, int field, float* host, uint64_t n);
int eq_batch_write_field(eq_batch* b, int64_t scene, int field, const float* host,
                         uint64_t n);
/* One field of every scene at once: dense size*size copies in scene order,
 * n = the sum of size*size (synchronous; one device-side layout conversion
 * and one device-to-host copy, fastest into pinned host memory). */
int eq_batch_read_fields(eq_batch* b, int field, float* host, uint64_t n);

/* `nframes` frames of every scene: one persistent kernel launch per frame
 * (thread blocks take scenes from a work queue, largest first), the whole
 * sequence captured once into a CUDA graph and replayed (the graph is kept
 * for the next call with the same nframes and tuning). Asynchronous. */
int eq_batch_step(eq_batch* b, int64_t nframes);
/* The same frames launched directly (no graph). */
int eq_batch_step_eager(eq_batch* b, int64_t nframes);
int eq_batch_synchronize(eq_batch* b);

/* One lin_solve (fluid.rs:301-325) of field x_field from x0_field on every
 * scene with each scene's sweep count, by the same block solver. */
int eq_batch_lin_solve(eq_batch* b, int mode, int x_field, int x0_field, float a, float c);

/* The other single phases on every scene (fields as in the eq_fluid_* forms):
 * diffuse (fluid.rs:276-298) with one `diffusion` for all scenes, project
 * (fluid.rs:330-375), advect (fluid.rs:378-432), set_boundaries
 * (fluid.rs:252-272). */
int eq_batch_diffuse(eq_batch* b, int mode, int x_field, int x0_field, float diffusion);
int eq_batch_project(eq_batch* b, int vx_field, int vy_field, int p_field, int div_field);
int eq_batch_advect(eq_batch* b, int mode, int d_field, int d0_field, int u_field,
                    int v_field);
int eq_batch_set_boundaries(eq_batch* b, int mode, int field);

/* Tuning: sweeps per wavefront pass (warps per thread block, 1..20; a
 * lin_solve of K sweeps takes ceil(K / sweeps_per_pass) passes) and thread
 * blocks per SM. The default is min(max K, 20) and 1. */
int eq_batch_set_tuning(eq_batch* b, int sweeps_per_pass, int blocks_per_sm);
int eq_batch_get_tuning(const eq_batch* b, int* sweeps_per_pass, int* blocks_per_sm);

/* Autotuner: times `trial_frames` frames for every candidate tuning from a
 * snapshot of the state (restored after each trial, so the simulation state
 * is unchanged), keeps the fastest. ms_out[q] (q < cap) receives candidate q's
 * ms per frame (0 if it does not fit); *ncand the candidate count. */
int eq_batch_autotune(eq_batch* b, int trial_frames, double* ms_out, int cap, int* ncand);

int eq_batch_get_stream(eq_batch* b, void** stream);
int eq_batch_launch_count(const eq_batch* b, uint64_t* count);

/* ---- the precision form: half-storage fluid ------------------------------ */

/* One scene whose six fields are STORED in FP16 or BF16 (half the bytes of
 * every field access) while every operation computes in FP32 on the widened
 * values. The frame keeps the reference's phases, order and array aliasing
 * (fluid.rs:437-524); the diffusion solves keep its lexicographic Gauss-Seidel
 * (`frames` sweeps, FP32 arithmetic). The two pressure solves (fluid.rs:
 * 353-362) are solved to a relative residual instead of a fixed sweep count:
 * mixed-precision iterative refinement with an FP32 residual, FP64 norms and a
 * multigrid correction stored in the half format. The solution's constant
 * (the pure-Neumann null space) is the one the refinement reaches from p = 0.
 * Results differ from the reference's by design; eq_hfluid_stats reports the
 * refinement and the post-projection divergence of the last frame. */
#define EQ_STORE_F16 1
#define EQ_STORE_BF16 2
/* Density and scratch stored in FP16, the four velocity fields (and the
 * pressure / divergence project keeps in them) in FP32, for batches and for
 * the precision form: advect's backtraces multiply a velocity's rounding by
 * dt*N cells, so FP16 velocities dominate the density error. */
#define EQ_STORE_F16_SCALARS 3

typedef struct eq_hstats {
  int32_t ir_iterations[2];  /* refinement rounds of the frame's two projects */
  double rel_residual[2];    /* final mean-free relative residual of each */
  double div_norm_before[2]; /* ||div v||_2 entering each project (FP64) */
  double div_norm[2];        /* ||div v||_2 after each project (FP64) */
} eq_hstats;

typedef struct eq_hfluid eq_hfluid; /* opaque */

/* Fluid::new (init() once, frame = DefaultWall) in half storage. Refinement
 * stops at a relative residual <= pressure_rtol or after max_refinements
 * rounds. */
int eq_hfluid_new(const eq_fluid_configs* fluid, const eq_simulation_configs* sim, int storage,
                  double pressure_rtol, int32_t max_refinements, int device, eq_hfluid** out);
int eq_hfluid_free(eq_hfluid* h); /* accepts NULL */
int eq_hfluid_fill_obstacle(eq_hfluid* h, int64_t x0, int64_t y0, int64_t x1, int64_t y1);
/* Sources applied at the start of the next step (add_density / add_velocity
 * order, fluid.rs:120-131). */
int eq_hfluid_add_sources(eq_hfluid* h, int64_t n, const uint32_t* x, const uint32_t* y,
                          const float* density, const float* vx, const float* vy);
int eq_hfluid_step(eq_hfluid* h); /* synchronises (the refinement loop reads its norms) */
int eq_hfluid_synchronize(eq_hfluid* h);
/* Dense size*size FP32 copies of a stored field (widened / rounded). */
int eq_hfluid_read_field(eq_hfluid* h, int field, float* host, uint64_t n);
int eq_hfluid_write_field(eq_hfluid* h, int field, const float* host, uint64_t n);
int eq_hfluid_stats(const eq_hfluid* h, eq_hstats* out);
int eq_hfluid_get_stream(eq_hfluid* h, void** stream);
int eq_hfluid_launch_count(const eq_hfluid* h, uint64_t* count);
/* Which diffusions of a step run on side streams (EQ_CONC_* bits, as
 * eq_fluid_set_concurrency; default both). */
int eq_hfluid_set_concurrency(eq_hfluid* h, int mask);
/* The kernel of the diffusion solves (eq_fluid_set_solver's values). */
int eq_hfluid_set_solver(eq_hfluid* h, int solver);

/* ---- the differentiation form: adjoint of the frame step --------------- */

/* No counterpart in the reference (its step has no derivative). A recorded
 * forward run of a plain handle and its reverse-mode derivative. The forward
 * is the handle's own bit-exact step: for f in [0, nframes), src[f] (a dense
 * size x size field, x fastest) is added to density and scratch at every cell
 * (add_density at each cell, fluid.rs:120-124), then step() (fluid.rs:437-524).
 * The state at every `checkpoint_every`-th frame is kept on the device;
 * backward() recomputes each segment from its checkpoint with the fields
 * every advect reads saved (the last segment keeps them from the forward
 * itself), and undoes it frame by frame with the adjoint
 * kernels (set_boundaries^T, reverse Gauss-Seidel sweeps, the transposed
 * bilinear scatter of advect, project^T), FP32 arithmetic. Gradients are
 * those of the reference's f32 step, including its discrete choices (advect's
 * row breaks and clamps) as the recorded run took them. The handle's configs
 * and mask must not change between forward and backward (EQ_ERR_STATE);
 * backward leaves the handle in the forward's final state. */
typedef struct eq_grad eq_grad; /* opaque; binds one eq_fluid, free it first */

int eq_grad_new(eq_fluid* h, int64_t max_frames, int64_t checkpoint_every, eq_grad** out);
int eq_grad_free(eq_grad* g); /* accepts NULL */
/* Runs nframes (<= max_frames) recorded frames from the handle's state.
 * src: nframes * size * size floats (host), or NULL for no sources (n = 0). */
int eq_grad_forward(eq_grad* g, int64_t nframes, const float* src, uint64_t n);
int eq_grad_forward_device(eq_grad* g, int64_t nframes, const float* d_src);
/* loss = 0.5 * sum over the interior of (density - target)^2 at the recorded
 * run's end (FP64 sum); seeds backward() with its adjoint. adj_density
 * (optional, host, size * size) receives density - target (0 on the frame). */
int eq_grad_l2_loss(eq_grad* g, const float* target, uint64_t n, double* loss,
                    float* adj_density);
/* adj_final: the adjoints of the six arrays after the run (6 * size * size,
 * EQ_FIELD_* order), or NULL to use the seed of eq_grad_l2_loss. Outputs
 * (each optional): grad_init, the adjoints of the six arrays before the run
 * (6 * size * size); grad_src, of every frame's source field
 * (nframes * size * size). Host pointers; synchronises. */
int eq_grad_backward(eq_grad* g, const float* adj_final, uint64_t n_adj, float* grad_init,
                     uint64_t n_init, float* grad_src, uint64_t n_src);
int eq_grad_backward_device(eq_grad* g, const float* d_adj_final, float* d_grad_init,
                            float* d_grad_src);
int eq_grad_frames(const eq_grad* g, int64_t* recorded);
/* Caps where the transposed Gauss-Seidel wavefront keeps its band of live
 * diagonals: 3 = spread over a cluster of 8 blocks (distributed shared
 * memory; the default where each block keeps >= 16 positions), 2 = one block,
 * y and its running sum in shared memory, 1 = y only, 0 = global memory;
 * -1 restores the default. */
int eq_grad_set_wavefront_storage(eq_grad* g, int max_store);
/* Caps the cluster form's barrier interval at max_m + 1 steps (0..3, same
 * default as the forward's), as eq_fluid_set_cluster_interval does there. */
int eq_grad_set_cluster_interval(eq_grad* g, int max_m);
/* The form the last transposed solve used (store as above) and its blocks. */
int eq_grad_get_wavefront_storage(const eq_grad* g, int* store, int* cluster_blocks);
/* With profiling on, every transposed Gauss-Seidel wavefront launch is
 * bracketed by CUDA events; kernel_stats returns (and clears) their total
 * device time and count. */
int eq_grad_set_profiling(eq_grad* g, int enable);
int eq_grad_kernel_stats(eq_grad* g, double* total_ms, uint64_t* launches);
int eq_grad_launch_count(const eq_grad* g, uint64_t* count);
/* The adjoint of one phase on host size x size arrays (in/out), at the bound
 * handle's mask and configs: set_boundaries, lin_solve (x_b -> adjoint before
 * the solve, x0_b accumulates), advect (at the forward state d0, u, v; d_b ->
 * adjoint of the old d; d0_b, u_b, v_b accumulate; distinct arrays), project
 * (p and div the aliased arrays, as in step()). */
int eq_grad_set_boundaries_adj(eq_grad* g, int mode, float* xb, uint64_t n);
int eq_grad_lin_solve_adj(eq_grad* g, int mode, float* xb, float* x0b, float a, float c,
                          uint64_t n);
int eq_grad_advect_adj(eq_grad* g, int mode, float* db, float* d0b, float* ub, float* vb,
                       const float* d0, const float* u, const float* v, uint64_t n);
int eq_grad_project_adj(eq_grad* g, float* vxb, float* vyb, float* pb, float* divb,
                        uint64_t n);

/* ---- lin_solve that allocates nothing ----------------------------------- */

/* No counterpart in the reference. lin_solve (the same kernels, the same
 * bit-exact result as eq_fluid_lin_solve) for callers that cannot allocate
 * device memory: a solver embedded in a host application that owns all device
 * memory through its own allocator or a fixed budget (a render engine, a
 * framework with a caching allocator) and does not let its plugins call
 * cudaMalloc; frame loops that must not take the device-wide synchronisation
 * cudaMalloc / cudaFree can cause (this call synchronises only `stream`).
 * The caller passes device pointers to x (in/out), x0 and the wall mask
 * (1 = DefaultWall, ghost frame all walls), each `size` rows with a row pitch
 * of `pitch` elements (pitch % 4 == 0, buffers 16-byte aligned), and the
 * stream to run on (NULL = legacy default stream).
 * All scratch lives in one static device array sized for
 * size <= 258 and pitch <= 288 (about 3.2 MB per GPU that loads the library,
 * held until exit); larger grids return EQ_ERR_ARG. The first call on a device
 * (that device current) looks the array up and clears it: make it before any
 * stream capture. Every call shares the array, which keeps the last call's
 * contents, so calls that overlap on the GPU race. Synchronises `stream`
 * after the mask check (EQ_ERR_ARG if the frame is not all walls, returned
 * before x is touched) and before returning (EQ_ERR_TIMEOUT from the device
 * error word; x is then undefined). */
int eq_lin_solve_noalloc(int mode, float* x, const float* x0, const uint8_t* cells,
                         uint32_t size, uint32_t pitch, int64_t iters, float a, float c,
                         void* stream);

/* ---- diagnostics ------------------------------------------------------- */

/* Device pointer of a field (pitched rows) and the row pitch in elements. */
int eq_fluid_device_field(eq_fluid* h, int field, float** dptr, uint32_t* pitch_elems);

/* Number of kernel launches this handle has issued since creation. */
int eq_fluid_launch_count(const eq_fluid* h, uint64_t* count);

/* Bounded-wait budget of the inter-block waits, in polling iterations
 * (default: about one second of polling). Lowering it makes a wait that
 * cannot complete end with EQ_ERR_TIMEOUT sooner. */
int eq_fluid_set_spin_limit(eq_fluid* h, int64_t iterations);

/* step() can run its independent phases side by side: EQ_CONC_VY puts the
 * vy diffusion, EQ_CONC_DENSITY the density diffusion on a side stream of the
 * handle, joined before its result is read (bit-exact: the same kernels on
 * the same data). 0 = one stream, in the reference's order. Default: both. */
#define EQ_CONC_VY 1
#define EQ_CONC_DENSITY 2
int eq_fluid_set_concurrency(eq_fluid* h, int mask);

/* Which kernel runs lin_solve (all are bit-exact).
 * 0 (default) = the strip wavefront (one launch per 20 sweeps over 32-row
 *   strips and groups of sweeps, blocks chained through tagged exports)
 *   wherever x, x0 and the codes are 16-byte aligned (the handle's own grids
 *   always are; its shared memory does not grow with N), else as 4.
 * 1 = the multi-block wavefront always.
 * 2 = the thread-block-cluster wavefront wherever it applies: 32 < N <= 1024
 *   (strips of up to 64 positions on at most 16 blocks), with its strips
 *   staged in shared memory whole where they fit (<= 32 sweeps, N up to
 *   ~320), else streamed through shared-memory rings (<= 31 sweeps).
 * 3 = the strip wavefront wherever it applies (as 0), else as 4.
 * 4 = the staged cluster form where it applies; the streamed form only for
 *   the solves step() runs on its side streams (it holds few SMs, so it
 *   runs beside the critical path's solve); else the multi-block wavefront.
 * get_solver reports the blocks per cluster of the cluster form (0 = it
 * does not apply); get_cluster_form its form: 0 = none, 1 = strips staged
 * whole, 2 = strips streamed. */
int eq_fluid_set_solver(eq_fluid* h, int solver);
int eq_fluid_get_solver(eq_fluid* h, int* cluster_blocks);
int eq_fluid_get_cluster_form(eq_fluid* h, int* form);
/* Caps the cluster wavefront's barrier interval at max_m + 1 steps (0..3;
 * by default 3 steps for N >= 192 and 2 below, the fastest measured; the
 * longest interval up to the cap that fits in shared memory is used). */
int eq_fluid_set_cluster_interval(eq_fluid* h, int max_m);
/* Sweep groups per strip of the strip wavefront: each strip's sweeps of one
 * launch are split over `groups` blocks (1..5; a block holds at most 10
 * sweeps, so 20 sweeps take at least 2 groups). 0 (default) = by grid size,
 * about one block per SM, except for the two velocity diffusions that step()
 * runs side by side (the fewest groups, so that both fit the SMs at once). */
int eq_fluid_set_strip_groups(eq_fluid* h, int groups);
/* Periods (of 4 wavefront steps) a strip-wavefront block waits, before its
 * first step, for the blocks it reads from to be ahead of it (0..64; 0 by
 * default). */
int eq_fluid_set_strip_slack(eq_fluid* h, int periods);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
 * work or events against the handle's launches. */
int eq_fluid_get_stream(eq_fluid* h, void** stream);

/* Kernel timing: while enabled, every lin_solve wavefront launch is bracketed
 * by CUDA events on the handle's stream. eq_fluid_kernel_stats synchronises,
 * returns the summed device time (ms) and the launch count since the last
 * reset, and resets. `kernel` 0 = the lin_solve wavefront. */
int eq_fluid_set_profiling(eq_fluid* h, int enable);
int eq_fluid_kernel_stats(eq_fluid* h, int kernel, double* total_ms, uint64_t* launches);

/* Message for the calling thread's last non-zero status ("" if none). */
const char* eq_last_error(void);

int eq_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* EQFLUID_H */
