/*
 * sphnj.h - C ABI of the GB300 particle-step library (libsphnj.so).
 *
 * This is the drop-in seam for SPHNJ's particle-step hot path.  The reference
 * has no plugin or FFI API of its own: its seam is the internal call
 * DeviceFunction::GPUCalulation(Sim*) (include/function.cuh:12,
 * src/calculation.cu:14-18), which reads the whole `Parameter` POD from the
 * __constant__ symbol `dev_par` and raw particle pointers from `dev_data`
 * (src/memory_copy.cu:5-11, include/data_pointer.cuh:48-116).  This header
 * replaces that seam with plain C: a POD mirror of `Parameter`, caller-owned
 * host SoA buffers, and an opaque context that owns every device allocation.
 *
 * Conventions
 *   - Every function returns an int status (SPHNJ_OK == 0) unless noted.
 *     No C++ exception crosses this boundary.
 *   - Host buffers are owned by the caller and only copied.
 *   - One context serves one host thread; each context launches on its own
 *     CUDA stream (or on the stream given to sphnj_set_stream).
 *   - Vectors are interleaved (x0 y0 x1 y1 ...), 2x2 matrices are stored
 *     column-major (m00 m10 m01 m11), i.e. the memory layout of
 *     Eigen::Vector2f/2d and Eigen::Matrix2f/2d that the reference uses.
 *   - Enumerations are 32-bit ints with the integer values of the
 *     reference's include/types.h:4-67.
 */
#ifndef SPHNJ_H
#define SPHNJ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SPHNJ_OK                0
#define SPHNJ_ERR_ARG           1   /* bad argument / NULL pointer          */
#define SPHNJ_ERR_IO            2   /* file missing or malformed            */
#define SPHNJ_ERR_CONFIG        3   /* required ini key missing (reference
                                       readParameter returned true)          */
#define SPHNJ_ERR_COUNT         4   /* .dat header count != line count      */
#define SPHNJ_ERR_CUDA          5   /* a CUDA runtime call failed           */
#define SPHNJ_ERR_CELL_OVERFLOW 6   /* a cell holds more than CELL_SIZE (64)
                                       particles: the reference's fixed
                                       64-slot lists would overflow
                                       (src/pair.cu:90-93, sort.cu:66-67)    */
#define SPHNJ_ERR_OUT_OF_GRID   7   /* a particle's cell id is outside the
                                       cell grid (the reference reads out of
                                       bounds there)                         */
#define SPHNJ_ERR_NONFINITE     8   /* NaN/Inf in a particle's position,
                                       velocity or density after an update
                                       (reported by the next synchronising
                                       call; the reference steps on)         */
#define SPHNJ_ERR_WATCHDOG      9   /* reserved for a bounded device wait
                                       that ran out: no kernel of this
                                       version waits on another, so none
                                       returns it                            */
#define SPHNJ_ERR_UNSUPPORTED  10   /* feature not available in this form   */
#define SPHNJ_ERR_NO_DEVICE    11   /* no CUDA device / extension missing   */

/* ---- enumerations (include/types.h:4-67) -------------------------------- */
enum { SPHNJ_LIQUID = 0, SPHNJ_GAS = 1 };                         /* PhaseType         */
enum { SPHNJ_SLIP = 0, SPHNJ_NO_SLIP = 1, SPHNJ_MOVING = 2 };     /* BoundaryType      */
enum { SPHNJ_SPLASH = 0, SPHNJ_FREE_SURFACE = 1,
       SPHNJ_VICINITY = 2, SPHNJ_INNER = 3 };                     /* FluidBoundaryType */
enum { SPHNJ_NO_PARTICLE = 0, SPHNJ_HAS_PARTICLE = 1,
       SPHNJ_HAS_NEAR_PARTICLE = 2 };                             /* NearParticle      */
enum { SPHNJ_LINEAR_ELASTIC = 0, SPHNJ_AUXETIC = 1 };             /* MaterialType      */
enum { SPHNJ_HYPER_ELASTIC = 0, SPHNJ_PLASTIC = 1 };              /* PlasticType       */
enum { SPHNJ_UNCONSTRAINED = 0, SPHNJ_FIXED = 1 };                /* SolidBoundaryType */
enum { SPHNJ_STRESS_2D = 0, SPHNJ_STRAIN_2D = 1 };                /* ConstitutionType  */
enum { SPHNJ_TRANSIENT = 0, SPHNJ_STEADY = 1 };                   /* TransientType     */

#define SPHNJ_CELL_SIZE 64            /* global.h:9 */

/* ---- parameters: POD mirror of the reference `Parameter` ---------------
 * Field groups follow include/physics.h:8-16, properties.h:7-54,
 * domain.h:7-21, sim_time.h:6-20 and kernel.h:6-31.  Values are derived by
 * sphnj_params_derive() with the reference formulas (kernel.cpp:25-41,
 * properties.cpp:53-89, domain.cpp:37-49, sim_time.cpp:27-32).            */
typedef struct sphnj_params {
    /* physics */
    float   gravity[2];                 /* (0, -gravity)  physics.cpp:12-14 */
    int32_t transient_type;
    /* fluid */
    int32_t fluid_number[2];            /* liquid, gas                      */
    int32_t fluid_number_total;
    float   sound_speed[2];
    float   reference_density[2];
    float   reference_density_inverse[2];
    float   gamma[2];
    float   viscosity[2];
    float   particle_shift_coef;
    float   gamma_inv[2];
    float   coefficient_p2rho[2];
    float   coefficient_rho2p[2];
    float   min_pressure;
    float   min_density[2];
    int32_t is_fluid_viscid;
    /* solid */
    int32_t solid_number;
    float   solid_reference_density;
    float   youngs_modulus;
    float   poisson_ratio;
    float   lambda;
    float   nu;                         /* shear modulus, named as in the reference */
    float   bulk_modulus;
    float   artificial_viscosity[2];    /* alpha, beta                       */
    float   solid_sound_speed;
    double  fixed_speed[2];
    int32_t constitution_type;
    int32_t plastic_type;
    float   auxetic_density;
    float   auxetic_modulus;
    float   auxetic_poisson_ratio;
    float   yield_strain;
    float   yield_stress;
    float   harden_strain;
    float   harden_coef;
    float   auxetic_lambda;
    float   auxetic_nu;
    /* virtual */
    int32_t virt_number;
    /* domain */
    float   cell_xmin[2];
    float   cell_xmax[2];
    float   domain_xmin[2];
    float   domain_xmax[2];
    int32_t cell_number[2];
    float   interval[2];
    float   interval_inv[2];
    int32_t cell_number_total;
    /* time */
    float   dt;
    int32_t istart;
    int32_t iend;
    int32_t solid_sub_step;
    int32_t shift_per_step;
    int32_t result_interval;
    int32_t sort_every_step;
    /* kernel */
    float   smoothing_length;
    float   particle_diameter;
    float   particle_volume;
    float   diameter_square;
    int32_t thread_num;
    float   smoothing_length_square;
    float   smoothing_length_inverse;
    float   smoothing_length_inverse_square;
    float   impact_length_hsml_ratio;
    float   impact_distance_square;
    float   kernel_coefficient_1;
    float   kernel_coefficient_2;
    float   kernel_differential;
    float   coefficient_3d_to_2d;
} sphnj_params;

/* ---- host state (caller-owned SoA; any pointer may be NULL) --------------
 * Upload: a NULL input field takes the reference's initial value
 * (include/host_data.cuh:24-115).  Download: only non-NULL fields selected
 * by the mask are written.  Counts are those of the params given to
 * sphnj_create.                                                           */
typedef struct sphnj_host_state {
    /* fluid (particle.cuh:20-32), n = fluid_number_total */
    float   *fluid_position;            /* 2n */
    float   *fluid_velocity;            /* 2n */
    float   *fluid_density;             /* n  */
    float   *fluid_pressure;            /* n  */
    int32_t *fluid_phase;               /* n  PhaseType                       */
    int32_t *fluid_boundary_type;       /* n  FluidBoundaryType               */
    int32_t *fluid_has_near_particle;   /* n  NearParticle                    */
    float   *fluid_du_dx;               /* 4n (column-major 2x2)              */
    float   *fluid_gradient;            /* 2n */
    float   *fluid_du_dt;               /* 2n */
    float   *fluid_color;               /* n  */
    float   *fluid_drho_dt;             /* n  */
    int32_t *fluid_cell_id;             /* n  (download only)                 */
    /* solid (particle.cuh:101-116), n = solid_number */
    double  *solid_position;            /* 2n */
    double  *solid_reference_position;  /* 2n */
    double  *solid_velocity;            /* 2n */
    int32_t *solid_boundary_type;       /* n  SolidBoundaryType               */
    int32_t *solid_material_type;       /* n  MaterialType                    */
    double  *solid_max_strain;          /* 4n */
    float   *solid_pressure;            /* n  */
    double  *solid_deformation;         /* 4n */
    double  *solid_stress_1st_piola;    /* 4n */
    double  *solid_correction;          /* 4n */
    double  *solid_du_dt;               /* 2n */
    float   *solid_normal;              /* 2n */
    float   *solid_couple_dudt;         /* 2n */
    int32_t *solid_cell_id;             /* n  (download only)                 */
    /* virtual (particle.cuh:184-192), n = virt_number */
    float   *virt_position;             /* 2n */
    float   *virt_normal;               /* 2n  NULL on upload: computed by the
                                           O(N_v^2) wall-normal pass before the
                                           first step (virt.cu:8-59)           */
    float   *virt_velocity;             /* 2n */
    float   *virt_pressure;             /* n  */
    float   *virt_density;              /* n  */
    int32_t *virt_phase;                /* n  */
    int32_t *virt_boundary_type;        /* n  BoundaryType                    */
    int32_t *virt_cell_id;              /* n  (download only)                 */
} sphnj_host_state;

/* field mask bits for sphnj_download */
#define SPHNJ_F_FLUID_KINEMATICS  (1u << 0)  /* position, velocity            */
#define SPHNJ_F_FLUID_THERMO      (1u << 1)  /* density, pressure, phase      */
#define SPHNJ_F_FLUID_FLAGS       (1u << 2)  /* boundary type, near flag      */
#define SPHNJ_F_FLUID_DERIVED     (1u << 3)  /* du_dx, gradient, du_dt, color, drho_dt */
#define SPHNJ_F_SOLID_KINEMATICS  (1u << 4)  /* position, reference position, velocity */
#define SPHNJ_F_SOLID_MATERIAL    (1u << 5)  /* boundary, material, max_strain */
#define SPHNJ_F_SOLID_DERIVED     (1u << 6)  /* pressure, F, P, L, du_dt, normal, couple */
#define SPHNJ_F_VIRT              (1u << 7)  /* all virtual fields            */
#define SPHNJ_F_CELL_IDS          (1u << 8)  /* per-particle cell ids         */
#define SPHNJ_F_ALL               0x1FFu

/* ---- forms ---------------------------------------------------------------- */
#define SPHNJ_FORM_PLAIN  0   /* reference precision (fluid FP32, solid FP64),
                                 reference cell-list order and stage order    */
#define SPHNJ_FORM_MIXED  1   /* mixed precision: FP32 in every pair loop;
                                 positions as integer cell + FP32 offset,
                                 integrated with Kahan compensation (fluid
                                 position and velocity; solid displacement
                                 and velocity); solids in total-Lagrangian
                                 displacement form with FP64 only for the 2x2
                                 correction-matrix inverse and the deformation
                                 gradient / PK1 stress step.  Same stages,
                                 lists and order as the plain form; results
                                 differ from it in rounding only.  The host
                                 state in and out is the plain layout (upload
                                 splits positions, download joins them). */

/* ---- host-side parameter and case I/O (no GPU needed) --------------------- */

/* Reads a flat ini file with the reference Config semantics (config.cpp:59-129,
 * config.h:122-159): `[section]` lines ignored, `#` starts a comment, later
 * keys override earlier ones, unknown keys ignored.  Fills every key the
 * reference reads, with its default (physics.cpp:12-17, properties.cpp:37-49,
 * properties.cpp:120-149, domain.cpp:10-18, sim_time.cpp:10-16,
 * kernel.cpp:11-14).  Returns SPHNJ_ERR_CONFIG when the reference's
 * readParameter would report failure (parameter.cpp:36-52). */
int sphnj_params_read_ini(const char *ini_path, sphnj_params *out);

/* Reads the three .dat headers under data_dir and checks the line counts
 * (Parameter::readParticleNumber, parameter.cpp:54-63,
 * properties.cpp:7-33,91-116,164-189). */
int sphnj_params_read_counts(const char *data_dir, sphnj_params *inout);

/* Derived constants (Parameter::initiateParameter, parameter.cpp:24-34). */
int sphnj_params_derive(sphnj_params *inout);

/* Parses fluid_particle.dat / solid_particle.dat / virt_particle.dat into the
 * caller's buffers (Fluid/Solid/Virtual_Host_List::addList,
 * host_data.cuh:24-115).  Fills position/velocity/density/pressure/phase for
 * fluid; position/velocity/reference/material/boundary for solid;
 * position/boundary for virtual.  Buffers must hold the counts in p. */
int sphnj_read_particles(const char *data_dir, const sphnj_params *p,
                         sphnj_host_state *out);

/* Byte layout check for foreign bindings: returns sizeof(sphnj_params),
 * sizeof(sphnj_host_state), sizeof(sphnj_diag), sizeof(sphnj_tuning) for
 * which = 0 / 1 / 2 / 3, else -1. */
int sphnj_abi_sizeof(int which);

/* ---- simulation context (GPU) --------------------------------------------- */
typedef struct sphnj_ctx sphnj_ctx;

/* Allocates all device memory for the counts in p (one arena).  Replaces
 * Sim::initiate + createCell + MemoryCopy::copyConstant (sim.cuh:27-33,
 * sim.cu:163-197, memory_copy.cu:8-12). */
int  sphnj_create(const sphnj_params *p, int form, sphnj_ctx **out);
void sphnj_destroy(sphnj_ctx *ctx);

/* Launch on the caller's stream (a cudaStream_t) instead of the context's
 * own stream; NULL restores the context's stream. */
int  sphnj_set_stream(sphnj_ctx *ctx, void *cuda_stream);

/* Copies a host state to the device (stream-ordered; returns after the copy
 * is complete).  Resets the cell lists to empty, as Cell() does
 * (cell.cuh:31-46), and sets the step counter to p->istart. */
int  sphnj_upload(sphnj_ctx *ctx, const sphnj_host_state *s);

/* Overwrites the fields selected by field_mask (SPHNJ_F_* groups) that are
 * non-NULL in s, in place: cell lists, step counter and every other field are
 * kept, so a driver can exchange particle data with other code between steps
 * (the reference's host code writes device state only at start-up,
 * sim.cu:40-60).  Returns after the copy is complete. */
int  sphnj_upload_fields(sphnj_ctx *ctx, uint32_t field_mask, const sphnj_host_state *s);

/* Advances n fluid steps; each is stages 3-10 of the reference loop
 * (calculation.cu:28-43: cell ids, sort every sort_every_step steps, cell
 * lists, solid coupling, virtual particles, fluid pair pass and update,
 * solid_sub_step solid sub-steps, max speed, shift_per_step shifting
 * passes).  Asynchronous: it returns once the work is queued.  Errors found
 * on the device are reported by the next synchronising call. */
int  sphnj_step(sphnj_ctx *ctx, int n);

/* Waits for the context's stream and reports device-side errors. */
int  sphnj_synchronize(sphnj_ctx *ctx);

/* Copies the selected fields to the caller's buffers (synchronous). */
int  sphnj_download(sphnj_ctx *ctx, uint32_t field_mask, sphnj_host_state *s);

/* Pinned host memory mapped into every device's address space, for the
 * arrays of a sphnj_host_state.  Fluid positions, velocities, densities and
 * pressures that lie in such memory (each array wholly inside one
 * allocation) are moved by sphnj_upload_fields and sphnj_download in one
 * kernel that reads or writes them in place over the host link, converting
 * the mixed form's cell + offset positions on the way, instead of one
 * copy-engine transfer per field plus a conversion pass.  Results are the
 * same either way; other memory takes the copy path.  Replaces the
 * reference's thrust host vectors (particle.cuh:65-81) as the host side of
 * its per-step copies.  Memory is zeroed.  sphnj_host_free takes only
 * pointers sphnj_host_alloc returned (SPHNJ_ERR_ARG otherwise); no transfer
 * may still use it. */
int  sphnj_host_alloc(uint64_t bytes, void **out);
int  sphnj_host_free(void *ptr);

/* sphnj_upload_fields(in_mask, in), sphnj_step(n) and sphnj_download(out_mask,
 * out) as one call, with the same results, returning when `out` is written
 * (in or out may be NULL: no upload or no download).  The host transfers
 * overlap the steps where the data allow: the fluid velocities, densities
 * and pressures go up on a second stream while the first step bins its
 * particles and builds its cell lists (its first stage that reads them
 * waits), and the last step's densities and pressures come down while its
 * shifting passes run (nothing after the fluid update changes them).  The
 * reference copies state to the host inside its loop every step for
 * getMaxSpeed and the global outputs (fluid.cu:429-440, output.cu:562-582),
 * with no overlap. */
int  sphnj_step_exchange(sphnj_ctx *ctx, int n, uint32_t in_mask, const sphnj_host_state *in,
                         uint32_t out_mask, sphnj_host_state *out);

/* Current step counter i (SimTime::i, sim_time.cpp:27-40). */
int  sphnj_get_step(const sphnj_ctx *ctx, int *step);

/* Cell lists for bit-exact comparison.  type: 0 fluid, 1 solid, 2 virtual.
 * start/count: cell_number_total ints each (may be NULL); list: the
 * concatenated per-cell lists, count[c] entries from start[c] (room for the
 * particle count of that type).  The per-cell order is the reference's
 * `particle_list` order for that type (pair.cu:66-154, sort.cu:59-92). */
int  sphnj_debug_cells(sphnj_ctx *ctx, int type, int32_t *start, int32_t *count,
                       int32_t *list, int32_t *n_listed);

/* Replaces the current cell lists of all three kinds (the reference's
 * Cell::particle_list contents, cell.cuh:11-25): per-cell counts
 * (cell_number_total ints) and the concatenated lists in cell order.  A NULL
 * count leaves that kind's lists empty.  With this and an uploaded state a
 * step can be resumed exactly from another implementation's snapshot. */
int  sphnj_debug_set_cells(sphnj_ctx *ctx,
                           const int32_t *count_fluid, const int32_t *list_fluid,
                           const int32_t *count_solid, const int32_t *list_solid,
                           const int32_t *count_virt, const int32_t *list_virt);

/* Sets the step counter i (SimTime::i) that the next step increments. */
int  sphnj_debug_set_step(sphnj_ctx *ctx, int step);

/* The max-speed value used by the last step's shifting passes
 * (getMaxSpeed, fluid.cu:429-440). */
int  sphnj_debug_max_speed(sphnj_ctx *ctx, float *max_speed);

/* Launch configuration of the fluid neighbour sweeps (pair pass and shifting
 * gradient): tiled != 0 stages the neighbours of a column segment of tile_h
 * cells (1..64) in shared memory per block; 0 runs one thread per particle.
 * Both sum the same terms in the same order: plain-form results are
 * identical, only the speed differs.  The mixed form takes neighbour
 * offsets in the frame of the tile's first cell (tiled) or of the particle's
 * own cell (one thread per particle), so tiling and tile height change its
 * results in rounding only.  Default: tiled, tile_h = 16. */
int  sphnj_set_tiling(sphnj_ctx *ctx, int tiled, int tile_h);

/* on != 0 (default): each kind of step (sort or rebuild step, list buffer,
 * first sort of the virtual particles) is captured once into a CUDA graph and
 * replayed, so a step costs one graph launch on the host; 0 launches every
 * kernel individually.  Results are identical.  Per-stage profiling
 * (sphnj_profile_enable) always launches individually. */
int  sphnj_set_graphs(sphnj_ctx *ctx, int on);

/* on != 0 (default): the kernels of a step are launched with programmatic
 * stream serialisation (programmatic dependent launch), so that each kernel's
 * blocks are scheduled while the previous kernel's last blocks still run and
 * wait on the device for its results; 0 launches them plainly, one after the
 * other.  Results are identical. */
int  sphnj_set_launch_chaining(sphnj_ctx *ctx, int on);

/* Tiled sweeps: on != 0 (default) stores per-step neighbour lists in the pair
 * pass for the shifting passes of the same step; 0 walks the 3x3 stencil in
 * every pass.  Results are identical.  sphnj_get_sweeps reports the current
 * configuration (any pointer may be NULL). */
int  sphnj_set_neighbour_lists(sphnj_ctx *ctx, int on);
int  sphnj_get_sweeps(const sphnj_ctx *ctx, int *tiled, int *tile_h, int *lists);

/* Threads per block of the tiled sweeps: the shifting passes (64, 128 or
 * 256) and the pair pass (128 or 256); 0 keeps each launch kind's default
 * (128 for a dense scene's shifting passes and pair pass, 256 for a sparse
 * scene's, 128 in batches).  Results are identical for every choice. */
int  sphnj_set_block_sizes(sphnj_ctx *ctx, int shift_threads, int pair_threads);
int  sphnj_get_block_sizes(const sphnj_ctx *ctx, int *shift_threads, int *pair_threads);

/* Autotuner of the sweep configuration (no counterpart in the reference,
 * whose launch shape is fixed at thread_num = 32).  Coordinate search over:
 * one thread per particle, or tiles of 8, 12, 16, 24, 32 cells with stored
 * neighbour lists and of 8, 16, 32 cells without; then the shifting passes'
 * block size (64, 128, 256 threads); then the pair pass's (128, 256).  For a
 * batch (sphnj_batch_autotune) the scenes with fluid are then split at their
 * median particle count into two size classes, and each class's tile height
 * is tuned with the other's fixed.  Each candidate runs `steps` steps from a
 * device copy of the current state (once to capture its graphs, once timed
 * with CUDA events); the state is put back after each trial, so tuning does
 * not advance or change the run (in the mixed form the installed tile height
 * then sets the rounding of later steps, as for sphnj_set_tiling).  The
 * fastest candidate is installed and
 * reported: tile_h / lists are those of class 0 (the only class of a single
 * scene); class_split is the fluid particle count at which class 1 starts
 * (0 with one class). */
typedef struct sphnj_tuning {
    int32_t tiled, tile_h, lists, candidates;
    double  ms_per_step;
    int32_t shift_block, pair_block;
    int32_t size_classes, class_split;
    int32_t class_tile_h[2], class_lists[2];
} sphnj_tuning;
int  sphnj_autotune(sphnj_ctx *ctx, int steps, sphnj_tuning *out);

/* ---- global diagnostics, reduced on the device in FP64 --------------------
 * The quantities of the reference's global outputs (output.cu:283-560),
 * which it computes on the host from full device->host copies of the state:
 * here one small device reduction, deterministic (fixed summation order),
 * no per-particle copy.  d = particle_diameter, dv = d^2, m = rho0[phase] dv. */
typedef struct sphnj_diag {
    int32_t step;              /* step counter when computed                  */
    int32_t n_liquid;          /* liquid particles counted for the front      */
    double  front;             /* max x over liquid + d/2 (outputEdge, output.cu:339-352); -1e300 without liquid */
    double  fluid_momentum[2]; /* sum m v                                     */
    double  fluid_kinetic;     /* sum m |v|^2 / 2                             */
    double  fluid_mass;        /* sum rho dv                                  */
    double  tip_disp[2];       /* x - X of the solid particle with the largest reference x
                                  (ties: closest to the mean reference y)    */
    double  solid_kinetic;     /* sum rho_s dv |v|^2 / 2 over reference x >= 0 (outputTotalEnergy, output.cu:426-455) */
    double  solid_strain;      /* sum (lambda/2 tr(E)^2 + mu E:E) dv, E = (F^T F - I)/2 (same)                     */
    double  total_force[2];    /* sum couple_dudt dv rho_material (outputTotalForce, output.cu:283-305)             */
    double  von_mises[2];      /* max von Mises stress of F^-1 P over LINEAR_ELASTIC, AUXETIC (output.cu:503-544)  */
    double  mean_pressure;     /* mean solid pressure (outputMeanPressure, output.cu:546-560)                     */
} sphnj_diag;
int  sphnj_diagnostics(sphnj_ctx *ctx, sphnj_diag *out);

/* Point probes (Probe::getData, probe.cu:7-119): Shepard-interpolated fluid
 * and solid velocity, pressure and density (solid density 0) at n points
 * xy[2n], written to out[4n] as vx vy p rho; a point with no neighbour gives
 * 0 0 0 rho0_liquid.  Each neighbour cell's own entries are used (the
 * reference indexes neighbour cells with the probe cell's counts). */
int  sphnj_probe(sphnj_ctx *ctx, int n, const float *xy, float *out);

/* ---- measurement (the reference has only a host clock() around its loop,
 * calculation.cu:24-46) -------------------------------------------------- */

/* Number of stages reported by sphnj_profile_read, and the name of each
 * (e.g. "fluid_pair", "shift_pass"). */
int  sphnj_profile_stage_count(void);
const char *sphnj_profile_stage_name(int stage);

/* on != 0: every later stage launch is bracketed by CUDA events recorded on
 * the launching stream; totals are reset. */
int  sphnj_profile_enable(sphnj_ctx *ctx, int on);

/* Synchronises, then returns per stage (arrays of sphnj_profile_stage_count()
 * entries, any may be NULL): accumulated device time in ms, number of timed
 * calls, and number of kernels those calls launched. */
int  sphnj_profile_read(sphnj_ctx *ctx, double *ms, int64_t *calls, int64_t *kernels);

/* Kernels launched by this context since it was created. */
int  sphnj_stat_launches(const sphnj_ctx *ctx, uint64_t *launches);

/* ---- cell-list rebuild without device allocation --------------------------
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc - code running while a host framework owns all
 * device memory through its own pool allocator, plugin hosts that forbid
 * allocation after start-up, real-time loops that must not enter the
 * driver's allocator - and so supply every buffer themselves.
 *
 * It performs one incremental cell-list rebuild of one particle kind, the
 * operation sphnj_step does on each step that is not a sort step
 * (fillCellList, pair.cu:66-154), with the same kernels and the same result:
 * from the previous lists and the particles' new cell ids, the new per-cell
 * lists in the reference's order.
 *
 * All pointers are device pointers owned by the caller:
 *   cell_id     [n_particles]       new cell id of each particle; every id
 *                                   must lie in 0..nx*ny-1 (not checked: an
 *                                   id outside it corrupts list_out)
 *   prev_range  [2*nx*ny]           previous {start, count} per cell (8-byte aligned)
 *   prev_list   [sum of counts]     previous lists, a valid CSR over 0..n_particles-1
 *   range_out   [2*nx*ny]           new {start, count} per cell (8-byte aligned)
 *   list_out    [n_particles]       new lists
 * As in the reference, a particle whose new cell is not one of the nine
 * around its previous cell (it moved more than one cell since the lists were
 * built) is dropped until the next sort: list_out then holds fewer than
 * n_particles entries (the sum of the new counts).
 * stream is a cudaStream_t (NULL = legacy default stream); the call only
 * enqueues work.  It allocates nothing: its scratch is a static device array
 * for at most SPHNJ_NOALLOC_MAX_CELLS cells (about 2.6 MB, held by every GPU
 * that loads the library until the process exits).  nx*ny above that limit
 * returns SPHNJ_ERR_UNSUPPORTED.  Each call outside a stream capture looks up
 * that array's device address in the current context (cudaGetSymbolAddress);
 * a call during a capture uses the address the last such call found on that
 * device, so make the first call on a device before any stream capture (a
 * first call inside a capture returns SPHNJ_ERR_ARG).  All calls share the one array, so calls that overlap
 * on the GPU (different streams, or different host threads) race and must
 * be serialised by the caller. */
#define SPHNJ_NOALLOC_MAX_CELLS 65536
int  sphnj_rebuild_cell_lists_noalloc(int nx, int ny, int n_particles, const int32_t *cell_id,
                                      const int32_t *prev_range, const int32_t *prev_list,
                                      int32_t *range_out, int32_t *list_out, void *stream);

/* Message of the last error on this context (never NULL). */
const char *sphnj_last_error(const sphnj_ctx *ctx);

/* ---- batches of independent scenes -----------------------------------------
 * The reference runs one case per process (main.cu:14-35).  A batch advances
 * many independent scenes - contexts created and uploaded as usual, of any
 * sizes and parameters - together: every stage of a step is one launch over
 * all of them, and each kind of step is replayed as one CUDA graph.  The
 * result for every scene is identical to stepping it alone.
 *
 * The scenes of a batch must share sort_every_step and be at the same step
 * (same istart, stepped together), and stay alive until the batch is
 * destroyed.  While in a batch a scene launches on the batch's stream, so its
 * uploads and downloads are ordered with the batch's steps; it may belong to
 * one batch at a time and must not be given another stream. */
typedef struct sphnj_batch sphnj_batch;

int  sphnj_batch_create(sphnj_ctx *const *scenes, int n, sphnj_batch **out);
void sphnj_batch_destroy(sphnj_batch *b);
int  sphnj_batch_set_stream(sphnj_batch *b, void *cuda_stream);
/* As sphnj_set_tiling / sphnj_set_graphs, for every scene of the batch. */
int  sphnj_batch_set_tiling(sphnj_batch *b, int tiled, int tile_h);
int  sphnj_batch_set_graphs(sphnj_batch *b, int on);
int  sphnj_batch_set_launch_chaining(sphnj_batch *b, int on);
int  sphnj_batch_set_neighbour_lists(sphnj_batch *b, int on);
int  sphnj_batch_get_sweeps(const sphnj_batch *b, int *tiled, int *tile_h, int *lists);
/* One scene's own sweep shape inside the batch (scene = its index in the
 * array given to sphnj_batch_create): the cells per tile and the list switch
 * of that scene; the batch's launches are shared, each scene sweeps tiles of
 * its own height.  Results are identical for every choice. */
int  sphnj_batch_set_scene_tiling(sphnj_batch *b, int scene, int tile_h, int lists);
int  sphnj_batch_get_scene_tiling(const sphnj_batch *b, int scene, int *tile_h, int *lists);
/* As sphnj_set_block_sizes, for the batch's launches. */
int  sphnj_batch_set_block_sizes(sphnj_batch *b, int shift_threads, int pair_threads);
/* As sphnj_autotune, over the whole batch (every scene copied and put back). */
int  sphnj_batch_autotune(sphnj_batch *b, int steps, sphnj_tuning *out);
/* Advances every scene n fluid steps (asynchronous, as sphnj_step). */
int  sphnj_batch_step(sphnj_batch *b, int n);
/* Waits for the batch's stream; reports the first scene with a device error. */
int  sphnj_batch_synchronize(sphnj_batch *b);
int  sphnj_batch_profile_enable(sphnj_batch *b, int on);
int  sphnj_batch_profile_read(sphnj_batch *b, double *ms, int64_t *calls, int64_t *kernels);
int  sphnj_batch_stat_launches(const sphnj_batch *b, uint64_t *launches);
const char *sphnj_batch_last_error(const sphnj_batch *b);

/* ---- checkpoint / restart ---------------------------------------------------
 * The reference has no checkpoint (it restarts only from its generated .dat
 * files).  A checkpoint holds the complete device state of a context - every
 * field, both cell-list buffers, the per-step neighbour lists and counters -
 * after a versioned header ("SPHNJCK1", form, step state, the parameters).
 * Loading it into a context created with the same particle counts, cell grid
 * and form continues the run bit-identically.  The host buffer variant takes
 * sphnj_checkpoint_size() bytes; the file variants write / read one file. */
int  sphnj_checkpoint_size(const sphnj_ctx *ctx, uint64_t *bytes);
int  sphnj_checkpoint_save(sphnj_ctx *ctx, void *buffer, uint64_t bytes);
int  sphnj_checkpoint_load(sphnj_ctx *ctx, const void *buffer, uint64_t bytes);
int  sphnj_checkpoint_write(sphnj_ctx *ctx, const char *path);
int  sphnj_checkpoint_read(sphnj_ctx *ctx, const char *path);

#ifdef __cplusplus
}
#endif

#endif /* SPHNJ_H */
