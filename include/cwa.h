/*
 * cwa.h — C ABI of the GB300 coupled SPH + wave-heightfield simulation step.
 *
 * The reference (VarunRamakri7/CoupledWaterAnimation) has no library ABI: its
 * step is a sequence of GLSL compute dispatches issued from idle()
 * (CoupledWaterAnimation/Main.cpp:530-562) over an SSBO of 64-byte particles
 * and a triple-buffered RGBA32F wave image.  Every entry point below replaces
 * one piece of that GL binding contract; the comment on each names the
 * reference code it stands in for.  All functions return a cwa_status and
 * never throw across the ABI.  Plain pointers and sizes only.
 *
 * Ownership: the library owns all device memory of a cwa_sim.  Host arrays
 * passed in are caller-owned and copied.  Device views are borrowed and stay
 * valid until the next cwa_step / pass call or cwa_destroy.
 *
 * Threading: one cwa_sim per host thread (no internal locking).  All work of a
 * sim runs on one CUDA stream owned by the sim; cwa_step and the pass calls
 * are asynchronous, downloads / reductions / cwa_synchronize block.
 */
#ifndef CWA_H
#define CWA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CWA_ABI_VERSION 1

typedef enum cwa_status {
  CWA_OK = 0,
  CWA_ERR_INVALID_ARG = 1, /* bad pointer, size, index or parameter          */
  CWA_ERR_OOM = 2,         /* device or pinned allocation failed             */
  CWA_ERR_CUDA = 3,        /* a CUDA runtime call failed                     */
  CWA_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up             */
  CWA_ERR_NONFINITE = 5,   /* a NaN/Inf particle position was met            */
  CWA_ERR_IO = 6,          /* checkpoint file could not be read or written   */
  CWA_ERR_NO_DEVICE = 7,   /* no CUDA device / driver                        */
  CWA_ERR_CAPACITY = 8,    /* size beyond a stated maximum                   */
  CWA_ERR_BOUNDS = 9       /* an index check of a debug build failed (the
                              access was skipped); release builds do not check */
} cwa_status;

/* Physics presets.
 * REFERENCE_3D: the shaders' own constants and rules
 *   (rho_pres_comp.glsl:49-81, force_comp.glsl:62-139,
 *    integrate_comp.glsl:56-178, wave_comp.glsl:171-206).
 * MULLER: the 3D Mueller-2003 SPH of the benchmark configurations (poly6
 *   density, spiky pressure gradient -45/(pi h^6), viscosity Laplacian,
 *   p = k(rho - rho0), reflective walls) with two-way particle<->heightfield
 *   coupling through fixed-point deposits. */
enum { CWA_PRESET_REFERENCE_3D = 0, CWA_PRESET_MULLER = 1 };

/* Accumulation precision of the density / force neighbour sums.
 * CWA_PREC_FP32: plain float sums.
 * CWA_PREC_COMPENSATED: cascaded compensated summation.  Pair terms are
 *   summed in float into short partials (one per candidate row for the
 *   density, one per group of pairs for the force), and each partial is
 *   folded into a Knuth two-sum accumulator.  The two-sum is applied to the
 *   partials, not to every pair term.
 * CWA_PREC_FP64: pair arithmetic and sums in double. */
enum { CWA_PREC_FP32 = 0, CWA_PREC_COMPENSATED = 1, CWA_PREC_FP64 = 2 };

/* std430 `struct Particle {vec4 pos, vel, force, extras;}`
 * (CoupledWaterAnimation/Main.cpp:167-173, rho_pres_comp.glsl:14-20).
 * extras = (rho, pressure, foam threshold, density coefficient). 64 bytes. */
typedef struct cwa_particle {
  float pos[4];
  float vel[4];
  float force[4];
  float extras[4];
} cwa_particle;

/* One independent scene.  Fields mirror the reference's uniform blocks:
 * ConstantsUniform (Main.cpp:184-190), BoundaryUniform (Main.cpp:192-198),
 * WaveUniforms (Main.cpp:200-204) and the shader #defines / consts. */
typedef struct cwa_scene_desc {
  int32_t preset;          /* CWA_PRESET_*                                    */
  int32_t n_particles;     /* NUM_PARTICLES                                   */
  int32_t wave_nx;         /* wave image width  (texture s axis = world x)    */
  int32_t wave_nz;         /* wave image height (texture t axis = world z)    */
  float box_lo[3];         /* BoundaryUniform.lower.xyz                       */
  float box_hi[3];         /* BoundaryUniform.upper.xyz                       */
  float cell_size;         /* uniform-grid cell edge in x and y; must be >= h */
  float cell_size_z;       /* cell edge in z; <= 0 means cell_size.  A finer
                              z edge (e.g. h/4) lets each particle scan only
                              the z-window its neighbours can occupy        */
  float mass;              /* ConstantsUniform.mass                           */
  float smoothing_length;  /* h = smoothing_coeff * PARTICLE_RADIUS           */
  float visc;              /* ConstantsUniform.visc                           */
  float rest_rho;          /* ConstantsUniform.resting_rho                    */
  float gas_const;         /* GAS_CONST (reference 4000; Mueller k)           */
  float dt;                /* SPH time step                                   */
  float gravity[3];        /* G                                               */
  float wall_restitution;  /* reference DAMPING 0.3; Mueller restitution     */
  float velocity_damping;  /* v *= 1 - velocity_damping*dt (reference 0.3)    */
  float particle_radius;   /* PARTICLE_RADIUS                                 */
  float crest_height;      /* CREST_THRESHOLD (reference only)                */
  float foam_speed;        /* |v| above which a particle turns to foam        */
  float wave_lambda;       /* WaveUniforms.attributes[0]                      */
  float wave_atten;        /* WaveUniforms.attributes[1]                      */
  float wave_beta;         /* WaveUniforms.attributes[2]                      */
  float wave_mode;         /* WaveUniforms.attributes[3]                      */
  float wave_uv_scale[2];  /* texture uv = pos.xz * scale + offset            */
  float wave_uv_offset[2];
  float surface_y0;        /* heightfield rest level (Mueller coupling)       */
  float surface_restitution; /* normal-push restitution (Mueller coupling)    */
  float couple_gain;       /* height change per unit deposited momentum       */
  int32_t deposit_shift;   /* deposit quantum = 2^-deposit_shift momentum     */
  int32_t flags;           /* reserved, must be 0                             */
} cwa_scene_desc;

typedef struct cwa_sim_options {
  int32_t device;          /* CUDA device ordinal                             */
  int32_t precision;       /* CWA_PREC_*                                      */
  int32_t use_graph;       /* capture cwa_step into CUDA graphs               */
  int32_t nb_threads;      /* threads per CTA of the neighbour passes; 0=auto */
  int32_t nb_stage;        /* density pass stages candidate rows in shared
                              memory: 0/1 = on (default), -1 = off         */
  float verlet_skin;       /* 0: sort and scan neighbours every step.  > 0:
                              keep the grid and a list of pairs within
                              h (1 + skin) until some particle has moved
                              skin h / 2 (needs cell_size >= h (1 + skin)) */
  int32_t nb_scan_minb;    /* density-scan kernel variant: min CTAs per SM
                              (4, 6, 8; 0 = 4)                              */
  int32_t nb_force_minb;   /* force kernel variant: min CTAs per SM (6, 8, 9;
                              0 = 9; FP64 runs 9 as 8)                      */
  int32_t wave_block;      /* blocked wave advance variant (CWA_WAVE_BLOCK_*)  */
  int32_t nb_queue;        /* 1: the density and force passes run as
                              persistent CTAs that take particle tiles from
                              a work queue (scenes with the most particles
                              first); 0: one CTA a tile (default).  Same
                              results either way.                          */
  int32_t reserved[2];
} cwa_sim_options;

/* Blocked wave advance variants: box of 128 x H cells (P: 256 x H) advanced
 * K steps per launch in shared memory; the R and P variants hold each
 * thread's box column (P: column pair) in registers and exchange only the
 * east / west neighbours through shared memory. */
enum {
  CWA_WAVE_BLOCK_32x4 = 0,  /* default: H 32, K 4 */
  CWA_WAVE_BLOCK_64x4 = 1,  /* H 64, K 4 */
  CWA_WAVE_BLOCK_64x8 = 2,  /* H 64, K 8 */
  CWA_WAVE_BLOCK_R32x4 = 3, /* registers, H 32, K 4 */
  CWA_WAVE_BLOCK_R64x4 = 4, /* registers, H 64, K 4 */
  CWA_WAVE_BLOCK_R64x8 = 5, /* registers, H 64, K 8 */
  CWA_WAVE_BLOCK_P32x4 = 6, /* registers, 256 x 32 box, two columns a thread, K 4 */
  CWA_WAVE_BLOCK_S32x4 = 7, /* registers, H 32, K 4, persistent CTAs that prefetch
                               their next box while walking the current one */
  CWA_WAVE_BLOCK_COUNT = 8
};

/* Borrowed device pointers of one scene, all in the current sorted order.
 * pos/vel/force are float4 arrays; rho_p is float2 (rho, pressure);
 * particle_id[i] is the upload index of sorted particle i. */
typedef struct cwa_device_view {
  int32_t n_particles;
  int32_t n_cells;
  int32_t grid_dims[3];
  int32_t wave_nx, wave_nz;
  float* pos;
  float* vel;
  float* force;
  float* rho_p;
  int32_t* particle_id;
  int32_t* cell_start;     /* n_cells + 1 entries, scene-local offsets        */
  float* wave_u_n;         /* current height field u^n                        */
  float* wave_u_nm1;       /* previous height field u^(n-1)                   */
  void* stream;            /* cudaStream_t of the sim                         */
} cwa_device_view;

typedef struct cwa_sim cwa_sim;

/* Indices into the cwa_reduce_totals output. */
enum {
  CWA_TOTAL_MASS = 0,
  CWA_TOTAL_MOMENTUM_X = 1,
  CWA_TOTAL_MOMENTUM_Y = 2,
  CWA_TOTAL_MOMENTUM_Z = 3,
  CWA_TOTAL_KINETIC = 4,
  CWA_TOTAL_POTENTIAL = 5,
  CWA_TOTAL_WAVE_VOLUME = 6,
  CWA_TOTAL_WAVE_ENERGY = 7,
  CWA_TOTALS_COUNT = 8
};

/* Passes of one step, in launch order (for cwa_get_pass_times). */
enum {
  CWA_PASS_GRID = 0,      /* hash + count + scan + stable insert + reorder */
  CWA_PASS_RHO_PRES = 1,
  CWA_PASS_FORCE = 2,
  CWA_PASS_INTEGRATE = 3,
  CWA_PASS_WAVE = 4,
  CWA_PASS_COUNT = 5
};

/* ---- misc --------------------------------------------------------------- */
const char* cwa_status_str(cwa_status s);
int32_t cwa_abi_version(void);
/* Last error text of this thread (CUDA error string or argument check). */
const char* cwa_last_error(void);

/* Fill a scene with a preset's constants.  REFERENCE_3D gives the values of
 * Main.cpp:28-35,184-204 and the shader consts; MULLER gives the benchmark
 * physics for lattice spacing `spacing` (h = 2s, m = rho0 s^3). */
cwa_status cwa_scene_defaults(int32_t preset, float spacing, cwa_scene_desc* out);
/* Set the wave grid size; for MULLER also re-derive lambda, beta, the uv
 * mapping over the box, the coupling gain and the deposit quantum. */
cwa_status cwa_scene_set_wave_grid(cwa_scene_desc* scene, int32_t nx, int32_t nz);
/* Uniform-grid dimensions ceil((hi-lo)/cell_size) per axis, in float32. */
cwa_status cwa_grid_dims(const cwa_scene_desc* scene, int32_t dims[3]);

/* ---- scene generators (host) ---------------------------------------------
 * make_cube: the reference's 64x5x64 lattice (Main.cpp:735-794).
 * dam_break: lattice dims[0..2] at `spacing` from box_lo + spacing/2, x
 *   fastest, jittered by U(-jitter*s, +jitter*s) per axis (seeded
 *   splitmix64 -> xoshiro256**), zero velocity.
 * bumps: sum of n_bumps Gaussians A~U(0.01,0.05), sigma~U(0.02,0.1),
 *   centre~U(0,1)^2 in texture uv, evaluated at texel centres. */
cwa_status cwa_make_reference_cube(const cwa_scene_desc* scene, cwa_particle* out, int32_t n);
cwa_status cwa_make_dam_break(const cwa_scene_desc* scene, const int32_t dims[3], float spacing,
                              float jitter, uint64_t seed, cwa_particle* out, int32_t n);
cwa_status cwa_make_bumps(const cwa_scene_desc* scene, int32_t n_bumps, uint64_t seed,
                          float* out_u, int32_t nx, int32_t nz);

/* ---- simulation lifecycle ------------------------------------------------
 * Replaces init_particles()/glBufferData (Main.cpp:764-794) and
 * StencilImage2DTripleBuffered::Init (StencilImage2DTripleBuffered.cpp:10-31). */
cwa_status cwa_create(const cwa_sim_options* opt, const cwa_scene_desc* scenes, int32_t n_scenes,
                      cwa_sim** out);
cwa_status cwa_destroy(cwa_sim* sim);
/* Host transfers return when the host buffer may be reused.  A page-locked
 * host buffer (cudaHostAlloc / cudaHostRegister) that is 16-byte aligned is
 * read or written by the library's kernels directly over the host link, in
 * coalesced 16-byte words; other buffers go through cudaMemcpyAsync.  The
 * bytes moved are the same either way. */
cwa_status cwa_upload_particles(cwa_sim* sim, int32_t scene, const cwa_particle* host, int32_t n);
cwa_status cwa_download_particles(cwa_sim* sim, int32_t scene, cwa_particle* host, int32_t n);
cwa_status cwa_upload_wave(cwa_sim* sim, int32_t scene, const float* u_n, const float* u_nm1,
                           int32_t nx, int32_t nz);
cwa_status cwa_download_wave(cwa_sim* sim, int32_t scene, float* u_n, float* u_nm1, int32_t nx,
                             int32_t nz);
/* StencilImage2DTripleBuffered::Reinit (StencilImage2DTripleBuffered.cpp:42-59):
 * wave_comp.glsl InitWave (MODE_INIT, :82-140) into both history buffers. */
cwa_status cwa_wave_reinit(cwa_sim* sim, int32_t scene);
/* StencilImage2DTripleBuffered::ReinitFromTexture (StencilImage2DTripleBuffered.cpp:61-77):
 * wave_comp.glsl InitFromImage (MODE_INIT_FROM_TEXTURE, :76-80) writes
 * u(x, y) = red(2x, y) / 255 of an RGBA8 texture, then the buffers rotate,
 * so u^n is the image field and u^(n-1) the old u^n.  `rgba` is host memory,
 * width x height texels of 4 bytes, row 0 = texture row 0 (the bottom row of
 * a bitmap loaded bottom-up, as the reference's loader does).  Texels past
 * the image read 0 (undefined in the shader).  Synchronous. */
cwa_status cwa_wave_init_from_image(cwa_sim* sim, int32_t scene, const uint8_t* rgba, int32_t width,
                                    int32_t height);

/* One full step per iteration: grid -> rho_pres -> force -> integrate -> wave
 * (idle(), Main.cpp:549-560, plus the uniform-grid sort).  Asynchronous. */
cwa_status cwa_step(cwa_sim* sim, int32_t n_steps);
/* The same passes one at a time (one glDispatchCompute each).  cwa_pass_grid
 * must precede rho_pres in every step; the wave pass ends the step. */
cwa_status cwa_pass_grid(cwa_sim* sim);
cwa_status cwa_pass_rho_pres(cwa_sim* sim);
cwa_status cwa_pass_force(cwa_sim* sim);
cwa_status cwa_pass_integrate(cwa_sim* sim);
cwa_status cwa_pass_wave(cwa_sim* sim);
/* n_steps wave passes over every scene's height field, with no particle
 * passes in between: the wave module stepped alone (Module::Compute in
 * StencilImage2DTripleBuffered.cpp:22-31 and wave_comp.glsl EvolveWave
 * :171-206, one dispatch per step).  Bit-identical to n_steps calls of
 * cwa_pass_wave; deposits pending from an integrate pass land in the first
 * step.  Steps run K at a time in shared memory (TMA-loaded tiles; K from
 * the sim's wave_block option), so device pointers of the wave buffers may
 * change: re-read cwa_get_device_view after it.  Asynchronous. */
cwa_status cwa_wave_advance(cwa_sim* sim, int32_t n_steps);
/* Wait for the sim's stream; report a device-side status (timeout, NaN). */
cwa_status cwa_synchronize(cwa_sim* sim);
cwa_status cwa_get_step_count(cwa_sim* sim, int64_t* steps);
/* Grid + Verlet-list rebuilds done by the device (Verlet mode). */
cwa_status cwa_get_rebuild_count(cwa_sim* sim, int64_t* rebuilds);
cwa_status cwa_get_device_view(cwa_sim* sim, int32_t scene, cwa_device_view* out);

/* Grid of the last grid build (every step, or the last Verlet rebuild):
 * cell_start (n_cells+1, scene-local) and sorted_id (upload index of each
 * sorted particle). */
cwa_status cwa_download_grid(cwa_sim* sim, int32_t scene, int32_t* cell_start, int32_t n_cells_p1,
                             int32_t* sorted_id, int32_t n);
/* Fixed-point deposits made by the last cwa_pass_integrate (before the wave
 * pass consumes and clears them): nx*nz int64 per scene. */
cwa_status cwa_download_deposits(cwa_sim* sim, int32_t scene, int64_t* out, int32_t nx, int32_t nz);

/* FP64 on-device totals of one scene (CWA_TOTAL_* order). */
cwa_status cwa_reduce_totals(cwa_sim* sim, int32_t scene, double out[CWA_TOTALS_COUNT]);

/* Versioned little-endian checkpoint of the sim's state + step count; a
 * resumed run is bit-identical to an uninterrupted one. */
cwa_status cwa_save(cwa_sim* sim, const char* path);
cwa_status cwa_load(cwa_sim* sim, const char* path);

/* Per-pass CUDA-event timing of the most recent step (ms), when enabled. */
cwa_status cwa_set_profiling(cwa_sim* sim, int32_t enable);
cwa_status cwa_get_pass_times(cwa_sim* sim, float* ms, int32_t n);
/* Test hook (fault injection on the host): with n >= 0, the n-th device
 * allocation of a cwa_sim from now on (counting from 0, process-wide) fails
 * with CWA_ERR_OOM, as if the device were out of memory; -1 turns it off.
 * Lets tests drive every allocation-failure path of cwa_create and of the
 * lazy allocations (wave advance scratch, the renderer's work buffers and
 * cube map) without exhausting a shared GPU. */
cwa_status cwa_debug_fail_alloc(int32_t n);
/* Number of kernels launched by the library on this sim since creation. */
cwa_status cwa_get_launch_count(cwa_sim* sim, int64_t* launches);

/* ---- autotuner ------------------------------------------------------------
 * Tries the neighbour-pass kernel variants on the sim's current state
 * (candidate staging on/off, launch-bound variants of the density scan and
 * force, 128- or 64-particle CTAs), each from the same snapshot for
 * trial_steps timed steps, keeps the fastest (unless it beats the options at
 * entry by less than 1.5%, which is within the trials' noise) and restores
 * the state.  It allocates a snapshot of the state while it runs. */
#define CWA_TUNE_MAX_TRIED 32
typedef struct cwa_tune_report {
  cwa_sim_options best;
  float best_ms;                 /* ms per step of the winner               */
  float entry_ms;                /* ms per step of the options at entry      */
  int32_t n_tried;
  cwa_sim_options tried[CWA_TUNE_MAX_TRIED];
  float tried_ms[CWA_TUNE_MAX_TRIED];
} cwa_tune_report;
cwa_status cwa_autotune(cwa_sim* sim, int32_t trial_steps, cwa_tune_report* out);
/* Times every blocked wave advance variant (CWA_WAVE_BLOCK_*) on the sim's
 * current wave state, each from the same snapshot for trial_steps wave steps
 * (rounded up to a multiple of 8, best of two rounds), keeps the fastest in
 * the sim's wave_block option and restores the state. */
typedef struct cwa_wave_tune_report {
  int32_t best;                               /* CWA_WAVE_BLOCK_*          */
  int32_t steps;                              /* timed wave steps / trial  */
  float ms_per_step[CWA_WAVE_BLOCK_COUNT];
} cwa_wave_tune_report;
cwa_status cwa_autotune_wave(cwa_sim* sim, int32_t trial_steps, cwa_wave_tune_report* out);
cwa_status cwa_get_options(cwa_sim* sim, cwa_sim_options* out);

/* ---- stand-alone operators on caller-owned device buffers ----------------
 * Exclusive prefix sum of int32 (replaces ParallelScan::Compute,
 * SphWave2D/ParallelScan.cpp:43-95 and prefix_sum_cs.glsl:18-43).  Any n >= 0
 * (the reference requires a power of two).  d_out may equal d_in.  The
 * workspace must hold cwa_scan_workspace_bytes(n) bytes of device memory.
 * The call is asynchronous on `stream`; its look-back waits are bounded, and
 * one that gives up (the output is then wrong) sets a status word in the
 * workspace, which cwa_scan_status reads. */
size_t cwa_scan_workspace_bytes(int32_t n);
cwa_status cwa_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int32_t n, void* d_workspace,
                                  size_t workspace_bytes, void* stream);
/* Waits for `stream`, then reports the last cwa_exclusive_scan_i32 that used
 * this workspace with this n: CWA_OK, or CWA_ERR_TIMEOUT when its look-back
 * gave up. */
cwa_status cwa_scan_status(int32_t n, const void* d_workspace, void* stream);

/* Exclusive scan that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot lend the workspace the scan above needs
 * and must not call cudaMalloc themselves (code inside a host application
 * that owns the whole device-memory budget, or real-time loops that cannot
 * risk the device synchronisation an allocation may cause).  The scan's
 * scratch is a fixed 66,048-byte array declared by the library, held on
 * every GPU that loads it until the process exits.  n above
 * CWA_NOALLOC_SCAN_MAX_N is rejected with CWA_ERR_CAPACITY.  A call made
 * outside a stream capture looks up the array's device address on the
 * current device; a call inside a capture reuses the last address found on
 * that device, so make one call on each device before any stream capture.
 * All calls on a device share the array: calls whose kernels overlap on the
 * GPU race (wrong sums, possibly a time-out, but no write outside the array),
 * so order them (e.g. one stream).  cwa_scan_noalloc_status waits for
 * `stream` and reports the last call on the current device: CWA_OK, or
 * CWA_ERR_TIMEOUT when its look-back gave up. */
#define CWA_NOALLOC_SCAN_MAX_N 16777216
cwa_status cwa_exclusive_scan_i32_noalloc(const int32_t* d_in, int32_t* d_out, int32_t n, void* stream);
cwa_status cwa_scan_noalloc_status(void* stream);

/* Uniform-grid build of n points (float4 xyz, stride 16 B): cell =
 * clamp(floor((p-lo)/cell), 0, dims-1), cell id (k*dims[1]+j)*dims[0]+i,
 * stable counting sort.  Replaces the COMPUTE_COUNTS / scan / INSERT
 * sequence of UniformGridSph2D::CollisionQuery (SphWave2D/UniformGridGpu2D.cpp:220-265)
 * and UniformGrid2D/ugrid_particles_cs.glsl:90-117, with a deterministic
 * (input-order) insert.  Outputs: d_cell_start (ncells+1), d_sorted_index (n),
 * optional d_cell_of (n, cell id of each input point, may be NULL). */
size_t cwa_grid_workspace_bytes(int32_t n, int32_t n_cells);
cwa_status cwa_grid_build(const float* d_pos4, int32_t n, const float lo[3], float cell_size,
                          const int32_t dims[3], int32_t* d_cell_start, int32_t* d_sorted_index,
                          int32_t* d_cell_of, void* d_workspace, size_t workspace_bytes,
                          void* stream);
/* Waits for `stream`, then reports the last cwa_grid_build on this
 * workspace with these sizes: CWA_OK, CWA_ERR_NONFINITE (a NaN/Inf point),
 * CWA_ERR_TIMEOUT (a scan look-back gave up) or CWA_ERR_CAPACITY (a cell
 * above 1024 points: that cell's order fell back to arrival order). */
cwa_status cwa_grid_status(int32_t n, int32_t n_cells, const void* d_workspace, void* stream);

/* ---- headless rendering (the reference's display(), Main.cpp:326-474) ----
 * One frame of the wave surface and the particles into an RGBA8 image, no
 * GL: skybox / surface (wave_vs.glsl, wave_fs.glsl over the strip mesh of
 * Surf.cpp) / particle sprites (particle_vs.glsl, particle_fs.glsl passes 0
 * and 2) with the depth test and SRC_ALPHA / ONE_MINUS_SRC_ALPHA blending
 * into an 8-bit colour target, fragments blended in draw order per pixel. */
typedef struct cwa_camera {
  float eye[3];     /* eye_persp, Main.cpp:138 */
  float center[3];  /* center_persp, Main.cpp:139 */
  float up[3];
  float fovy;       /* radians (glm::perspective, Main.cpp:348) */
  float near_z, far_z;
} cwa_camera;

typedef struct cwa_render_params {
  int32_t width, height;
  float angle;           /* model rotation about y (Main.cpp:153) */
  float particle_scale;  /* Main.cpp:154 */
  float wave_scale;      /* Main.cpp:155 */
  float point_size;      /* sprite edge in pixels (glPointSize, Main.cpp:913) */
  int32_t surface_res;   /* strip mesh vertices per side (WAVE_RES, Main.cpp:29) */
  int32_t draw_surface;  /* drawSurface, Main.cpp:162 */
  int32_t draw_particles;/* drawParticles, Main.cpp:163 */
  int32_t draw_skybox;   /* 1: the cube map behind everything (see cwa_render) */
  int32_t reserved[4];
} cwa_render_params;

/* The reference's startup view (Main.cpp:138-165, 913): eye (7, 4, 0),
 * centre (0, -1, 0), 45-degree field of view, near 0.1, far 100, angle 0.75,
 * particle scale 5, wave scale 0.047, 8-pixel sprites, a 512-vertex strip
 * mesh, surface and particles drawn, skybox behind off. */
cwa_status cwa_render_defaults(int32_t width, int32_t height, cwa_camera* camera, cwa_render_params* params);
/* The environment cube map (LoadCubemap, LoadTexture.cpp:35-67): six
 * face_size x face_size RGBA8 faces in the order +x, -x, +y, -y, +z, -z,
 * rows top-down as stored in the image files.  Without one, cube-map
 * lookups read (0, 0, 0, 1). */
cwa_status cwa_render_set_skybox(cwa_sim* sim, const uint8_t* faces_rgba, int32_t face_size);
/* Render one frame of `scene` into host memory (width * height * 4 bytes,
 * row 0 = the bottom row, as glReadPixels returns it).  Departures, by
 * design: particle normals come from this frame's depth image (the
 * reference reads last frame's); the skybox, drawn at depth 1.0 and
 * rejected by the default GL_LESS test against the cleared depth, appears
 * only with draw_skybox = 1; triangles with a vertex outside the near/far
 * planes or behind the eye are dropped instead of clipped.  Synchronous.
 * The frame's device work buffers stay with the sim and only grow, so
 * frames of a size already rendered allocate no device memory. */
cwa_status cwa_render(cwa_sim* sim, int32_t scene, const cwa_camera* camera, const cwa_render_params* params,
                      uint8_t* out_rgba);

/* ---- the 2D solver family (SphWave2D) ----
 * The reference's 2D predecessor: cubic-spline SPH (SphWaveKoschier2D_grid_cs.glsl)
 * with signed-distance walls over a 32 x 32 uniform grid (SphUgrid,
 * StencilBuffer.cpp:138-179, two substeps of grid build + density + forces
 * per frame), coupled one way to a 1D shallow-water field advanced by a
 * two-phase Lax-Wendroff step (Shallow1D_cs.glsl, ImageStencil::Compute,
 * StencilImage2D.cpp:141-163).  Each frame runs the SPH substeps on the
 * field of the previous frame, then the wave step (SphWave2D/Main.cpp:220-241). */
typedef struct cwa2d_particle {
  float pos[4];  /* x, y, 0, enabled (1) / disabled (0) */
  float vel[4];  /* vx, vy, 0, pressure */
  float acc[4];  /* ax, ay, 0, density */
} cwa2d_particle;  /* SphWave2D Particle, Main.cpp:34-39 (48 bytes) */

typedef struct cwa2d_params {
  int32_t n_particles;    /* num_particles = 32*128 (Main.cpp:41) */
  int32_t wave_cells;     /* 128 (Main.cpp:89) */
  int32_t sph_substeps;   /* 2 (Main.cpp:302) */
  int32_t wave_substeps;  /* 1 (StencilImage2D.h:55) */
  int32_t grid_cells[2];  /* 32 x 32 (StencilBuffer.cpp:138) */
  int32_t init_columns;   /* WIDTH = 128, the initial lattice's columns */
  float view_size[2];     /* VIEW_WIDTH, VIEW_HEIGHT = 9.6 */
  float particle_radius;  /* 0.025; support H = 4 r */
  float rest_density;     /* 1000 */
  float visc;             /* 0.05 */
  float dt;               /* 0.002 */
  float gas_const;        /* 35000 (weakly compressible, gamma 3) */
  float bottom;           /* 0.3: floor plane offset */
  float wave_lambda;      /* 0.001 (Shallow1D_cs.glsl:23); Wave1D: 0.01 (Wave1D_cs.glsl:21) */
  float wave_dx;          /* 0.1 (shallow water only) */
  int32_t wave_kind;      /* CWA2D_WAVE_SHALLOW (default) or CWA2D_WAVE_1D */
  float wave_atten;       /* Wave1D attenuation 0.9995 (Wave1D_cs.glsl:22) */
  float wave_beta;        /* Wave1D damping 0.001 (Wave1D_cs.glsl:23) */
  int32_t reserved[1];
} cwa2d_params;

/* The 1D field the SPH samples.  CWA2D_WAVE_SHALLOW: Shallow1D_cs.glsl, two
 * buffers, cells (h, uh, h_half, uh_half), the app's active choice
 * (InitShallowWaterEquation, SphWave2D/Main.cpp:77-97).  CWA2D_WAVE_1D:
 * Wave1D_cs.glsl, the damped wave equation on three buffers with free
 * boundaries, cells (h, velocity, acceleration, 0); the app's
 * InitWaveEquation (Main.cpp:63-75) runs it on 1024 cells with 10 substeps
 * and lambda 0.01. */
enum { CWA2D_WAVE_SHALLOW = 0, CWA2D_WAVE_1D = 1 };

typedef struct cwa2d_sim cwa2d_sim;
enum {
  CWA2D_PASS_GRID = 0,          /* uniform grid of the current positions */
  CWA2D_PASS_DENSITY = 1,       /* MODE_COMPUTE_DENSITY_PRESSURE */
  CWA2D_PASS_FORCE = 2,         /* MODE_COMPUTE_FORCES (integrates) */
  CWA2D_PASS_WAVE_PREDICT = 3,  /* Shallow1D MODE_ITERATE0 */
  CWA2D_PASS_WAVE_CORRECT = 4,  /* Shallow1D MODE_ITERATE1 */
  CWA2D_PASS_WAVE_ITERATE = 5   /* Wave1D MODE_ITERATE */
};

cwa_status cwa2d_defaults(cwa2d_params* out);
cwa_status cwa2d_create(const cwa2d_params* params, int32_t device, cwa2d_sim** out);
cwa_status cwa2d_destroy(cwa2d_sim* sim);
/* InitParticle (MODE_INIT) and the wave's ImageStencil::Reinit: Shallow1D
 * MODE_INIT_0, or Wave1D MODE_INIT_0 then MODE_INIT_1. */
cwa_status cwa2d_reinit(cwa2d_sim* sim);
/* The "Splash" button (ImageStencil::ComputeFunc(1)): MODE_INIT_1 on the
 * current field. */
cwa_status cwa2d_splash(cwa2d_sim* sim);
/* n frames (SPH substeps, then the wave substeps), one CUDA graph each. */
cwa_status cwa2d_step(cwa2d_sim* sim, int32_t n_steps);
/* One pass of a frame (CWA2D_PASS_*), eager; density needs a grid pass first. */
cwa_status cwa2d_pass(cwa2d_sim* sim, int32_t pass);
cwa_status cwa2d_upload_particles(cwa2d_sim* sim, const cwa2d_particle* host, int32_t n);
cwa_status cwa2d_download_particles(cwa2d_sim* sim, cwa2d_particle* host, int32_t n);
/* The newest wave field: n cells of 4 floats (see CWA2D_WAVE_*). */
cwa_status cwa2d_upload_wave(cwa2d_sim* sim, const float* cells4, int32_t n);
cwa_status cwa2d_download_wave(cwa2d_sim* sim, float* cells4, int32_t n);
/* CWA2D_WAVE_1D only: the field one step older (the iteration's c1). */
cwa_status cwa2d_upload_wave_prev(cwa2d_sim* sim, const float* cells4, int32_t n);
cwa_status cwa2d_download_wave_prev(cwa2d_sim* sim, float* cells4, int32_t n);
cwa_status cwa2d_synchronize(cwa2d_sim* sim);

/* ---- position-based box collisions on the uniform grid ----
 * The reference's GridTestPbdGpu3D demo (UniformGrid2D/UniformGridGpu3D.cpp:
 * 292-350 and uniform_grid_pbd_3D_cs.glsl): axis-aligned boxes inserted into
 * every grid cell they overlap, one Jacobi PBD iteration per substep
 * (PreAnimate, collision query against the extents and the other boxes with
 * friction, PostAnimate with SOR factor k and restitution e).  The shader
 * accumulates every constraint with float atomics, so its sums depend on
 * thread order; here each box gathers its contributions in a fixed order
 * (partners by index), which makes a step deterministic. */
typedef struct cwa_pbd_box {
  float color[4];  /* (1, 1, 1, 1), red (1, 0, 0, 1) after a contact */
  float x[4];      /* position, w = 1 */
  float v[4];      /* velocity */
  float p[4];      /* predicted position */
  float dp_t[4];   /* friction displacement sum */
  float dp_n[4];   /* normal displacement sum */
  float hw[4];     /* half widths */
  float rm;        /* 1 / mass = 1 / (hw.x hw.y hw.z) */
  float n;         /* constraint count */
  float e;
  float padding;
} cwa_pbd_box;  /* PbdObj, UniformGridGpu3D.h:27-39 (128 bytes) */

typedef struct cwa_pbd_params {
  int32_t n_boxes;      /* 4 * 1024 (UniformGrid2D/Main.cpp:49) */
  int32_t grid_cells[3];/* 16^3 over the extents (UniformGridGpu3D.cpp:292) */
  float extents_lo[3], extents_hi[3];  /* [-1, 1]^3 */
  float g[3];           /* (0, -0.1, 0) (UniformGridGpu3D.h:45-55) */
  float dt;             /* 0.02 */
  float damping;        /* 0.999 */
  float k;              /* SOR factor 1.75 */
  float k_static;       /* 10 */
  float sleep_thresh;   /* 0.0005 */
  float mu_k, mu_s;     /* 0.4, 0.5 */
  float e;              /* restitution 0.75 */
  int32_t substeps;     /* 1 */
  int32_t max_contacts; /* contact slots per box (0 = 64); more in one step is CWA_ERR_CAPACITY */
  int32_t reserved[3];
} cwa_pbd_params;

typedef struct cwa_pbd_sim cwa_pbd_sim;
cwa_status cwa_pbd_defaults(cwa_pbd_params* out);
/* GridTestPbdGpu3D::Init (UniformGridGpu3D.cpp:299-336): positions
 * 0.5 U(-1, 1)^3, velocities 0.1 U(-1, 1)^3, half widths U(0.15, 0.45) cell
 * edges per axis, drawn from the library's seeded generator. */
cwa_status cwa_pbd_make_boxes(const cwa_pbd_params* params, uint64_t seed, cwa_pbd_box* out, int32_t n);
cwa_status cwa_pbd_create(const cwa_pbd_params* params, int32_t device, cwa_pbd_sim** out);
cwa_status cwa_pbd_destroy(cwa_pbd_sim* sim);
cwa_status cwa_pbd_upload(cwa_pbd_sim* sim, const cwa_pbd_box* host, int32_t n);
cwa_status cwa_pbd_download(cwa_pbd_sim* sim, cwa_pbd_box* host, int32_t n);
/* n frames of Animate (UniformGridGpu3D.cpp:338-346): substeps x
 * (grid build, PreAnimate, collision query, PostAnimate). */
cwa_status cwa_pbd_step(cwa_pbd_sim* sim, int32_t n_steps);
/* Contact pairs found by the last collision query. */
cwa_status cwa_pbd_pair_count(cwa_pbd_sim* sim, int64_t* pairs);

#ifdef __cplusplus
}
#endif
#endif /* CWA_H */
