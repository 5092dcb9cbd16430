/*
 * fsim.h -- C ABI of the GB300 (sm_103a) fluid-simulation step library.
 *
 * One fsim_ctx owns a MAC grid, a particle set, the obstacle list and one CUDA
 * stream on the current device.  It replaces the per-step path of the
 * reference simulator (dkiovics/fluid_simulator, src/Simulator/simulator):
 * Simulator::simulate (simulator.cpp:51-100) and the MacGrid /
 * BridsonSolverGrid / HashedParticles state it runs on.  All calls are
 * single-caller per context and stream-ordered; every function returns 0 or a
 * negative FSIM_E_* code, and fsim_last_error() describes the last failure.
 * No C++ exception crosses this boundary.
 *
 * Conventions
 *   * Host arrays are FP32 AoS per particle: pos[3n], vel[3n], c[9n] where
 *     c[9i + 3a + b] is component b of the APIC vector c[a] of particle i (the
 *     reference's Particle::c, particle.h:8-12).
 *   * Grid fields are exchanged in the reference's cell order, x-major with z
 *     fastest: index (x*ny + y)*nz + z (MacGrid::cell, macGrid.h:91-93).  Face
 *     field a of cell (x,y,z) is the face on the +a side of that cell
 *     (MacGridCell::faces, macGrid.cpp:25-27).
 *   * `where` selects host (FSIM_HOST) or device (FSIM_DEVICE) memory for the
 *     caller's buffer; device buffers are only borrowed for the duration of the
 *     call (the copy is stream-ordered and complete when the call returns).
 */
#ifndef FSIM_H
#define FSIM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSIM_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define FSIM_OK 0
#define FSIM_E_INVALID (-1)       /* bad argument or unsupported combination */
#define FSIM_E_OOM (-2)           /* device or host allocation failed */
#define FSIM_E_CUDA (-3)          /* CUDA runtime/driver error */
#define FSIM_E_NOT_CONVERGED (-4) /* reserved: the step itself reports convergence in stats */
#define FSIM_E_NAN (-5)           /* non-finite solver scalar */
#define FSIM_E_TIMEOUT (-6)       /* a bounded device-side wait gave up */
#define FSIM_E_UNSUPPORTED (-7)   /* feature not built (see fsim_last_error) */
#define FSIM_E_STATE (-8)         /* call out of order (e.g. G2P before P2G) */
#define FSIM_E_CAPACITY (-9)      /* input larger than a fixed capacity (fsim_p2g_noalloc) */

/* ---- enums ------------------------------------------------------------- */
enum fsim_transfer { FSIM_PIC = 0, FSIM_FLIP = 1, FSIM_APIC = 2 }; /* Simulator::P2G2PType */
enum fsim_cell { FSIM_WATER = 0, FSIM_AIR = 1, FSIM_SOLID = 2 };   /* MacGridCell::CellType */
enum fsim_where { FSIM_HOST = 0, FSIM_DEVICE = 1 };

enum fsim_obstacle_type {
    FSIM_OBS_SPHERE = 0,      /* SphericalObstacle (obstacles.hpp:36-44) */
    FSIM_OBS_BOX = 1,         /* RectengularObstacle (obstacles.hpp:26-34) */
    FSIM_OBS_SOURCE = 2,      /* SphericalParticleSource (obstacles.hpp:46-57) */
    FSIM_OBS_SINK = 3,        /* SphericalParticleSink (obstacles.hpp:59-65) */
    FSIM_OBS_DISC_SOURCE = 4, /* extension: horizontal disc emitting 8 jittered particles
                                 per covered cell per step (no reference counterpart) */
    FSIM_OBS_BOX_SINK = 5     /* extension: axis-aligned box deleting particles */
};

/* Convergence test of the pressure solve. */
enum fsim_tol_mode {
    FSIM_TOL_ABS_MAX = 0, /* max_i |r_i| < tol: the reference's test (bridsonSolverGrid.cpp:276-281) */
    FSIM_TOL_REL_L2 = 1   /* ||r||_2 <= tol * ||b||_2 */
};

/* Arithmetic of the pressure solve. */
enum fsim_precision {
    FSIM_PREC_MIXED = 0, /* FP32 vectors/stencils/preconditioner, FP64 dots and scalars,
                            FP64 solution with FP64 true-residual replacement */
    FSIM_PREC_FP32 = 1,  /* as MIXED but the solution and residual stay FP32 */
    FSIM_PREC_FP64 = 2   /* all-FP64 PCG (precision-study oracle on the device) */
};

/* Preconditioner of the pressure solve. */
enum fsim_precond {
    FSIM_PRECOND_RBIC = 0, /* incomplete Cholesky in red-black order (modified, tau 0.97) */
    FSIM_PRECOND_MG = 1    /* geometric multigrid V-cycle (red-black Gauss-Seidel smoothing) */
};

/* Incompressibility solver, SimulationConfig::gridSolverType (simulationManager.cpp:16-19). */
enum fsim_grid_solver {
    FSIM_SOLVER_PCG = 0, /* BridsonSolverGrid: pressure PCG (bridsonSolverGrid.cpp:244-293) */
    FSIM_SOLVER_SOR = 1  /* BasicMacGrid: max_iters red-black SOR sweeps on the face velocities,
                            over-relaxation 1.98 (basicMacGrid.cpp:5-88) */
};

/* Initial guess of the pressure solve. */
enum fsim_warm_start {
    FSIM_WARM_ZERO = 0,     /* p0 = 0, as the reference */
    FSIM_WARM_PREVIOUS = 1, /* previous step's pressure */
    FSIM_WARM_GUESS = 2,    /* fsim_set_pressure_guess, falling back to the previous step's
                               pressure when the guess has the larger residual */
    FSIM_WARM_LEARNED = 3,  /* the attached warm-start network (fsim_set_net), falling back
                               to the previous step's pressure when its guess has the larger
                               residual */
    FSIM_WARM_LEARNED_RESIDUAL = 4 /* the previous step's pressure plus the network's answer to
                               the residual that pressure leaves (b - A p_prev, the same kind of
                               Poisson problem), falling back to the previous pressure alone
                               when the sum has the larger residual */
};

/* Step stages, in the order Simulator::simulate runs them (simulator.cpp:51-100). */
enum fsim_stage {
    FSIM_STAGE_SPAWN = 0,
    FSIM_STAGE_ADVECT = 1,
    FSIM_STAGE_PUSH_APART = 2, /* HashedParticles::pushParticlesApart (hashedParticles.cpp:64-107) with
                                  deterministic Jacobi semantics (see push_apart_enabled) */
    FSIM_STAGE_PUSH_OUT = 3,
    FSIM_STAGE_STOP = 4,
    FSIM_STAGE_P2G = 5,       /* sort by cell + resetGridValues + p2gTransfer + marking */
    FSIM_STAGE_MARK = 6,      /* fused into FSIM_STAGE_P2G (no-op) */
    FSIM_STAGE_OBSTACLES = 7,
    FSIM_STAGE_WALLS = 8,
    FSIM_STAGE_POST_P2G = 9,
    FSIM_STAGE_SOLVE = 10,
    FSIM_STAGE_EXTRAPOLATE = 11,
    FSIM_STAGE_G2P = 12,
    FSIM_NUM_STAGES = 13
};

/* Grid fields for fsim_get_grid / fsim_set_grid. */
enum fsim_field {
    FSIM_F_FLAGS = 0,   /* uint8 fsim_cell */
    FSIM_F_AVGPNUM = 1, /* float: particle density (MacGridCell::avgPNum) */
    FSIM_F_VX = 2, FSIM_F_VY = 3, FSIM_F_VZ = 4,    /* float face v (after P2G/obstacles/walls) */
    FSIM_F_V2X = 5, FSIM_F_V2Y = 6, FSIM_F_V2Z = 7, /* float face v2 */
    FSIM_F_PRESSURE = 8, /* float: last solved pressure, 0 outside fluid */
    FSIM_F_COUNT = 9,    /* int32: particles per cell from the last sort */
    FSIM_F_DIVERGENCE = 10 /* float: pressure right-hand side of the last solve */
};

/* ---- structs ----------------------------------------------------------- */

/* MacGrid(targetDimensions, resolution, twoD) (macGrid.h:28). */
typedef struct fsim_grid_desc {
    double dims[3];    /* target dimensions */
    double resolution; /* cells per unit length (rounded to float as BridsonSolverGrid does) */
    int two_d;         /* 2D mode: z is 3 cells of dims[2] / 3, particles stay on z = dims[2] / 2,
                          G2P sets v.z = 0 (macGrid.cpp:9-13, simulator.cpp:382-385) */
} fsim_grid_desc;

/* Simulator::SimulatorConfig (simulator.h:30-39) + MacGrid public fields
 * (macGrid.h:173-179) + the particle radius + solver controls. */
typedef struct fsim_params {
    int transfer;           /* fsim_transfer */
    float flip_ratio;
    float gravity;          /* signed, added to v_y * dt */
    int gravity_enabled;
    int push_apart_enabled; /* SimulatorConfig::pushApartEnabled: after advection every particle
                               moves by the sum of half-overlaps with all particles within 2r
                               (positions from before the pass), then is clamped; the reference's
                               in-place pairwise update is racy, this is its deterministic form.
                               Needs particle_r <= h/2. */
    int spawning_enabled;
    int despawning_enabled;
    int stop_particles;
    int top_solid;          /* isTopOfContainerSolid */
    int pressure_enabled;   /* density-correction term in the rhs */
    double pressure_k;
    double average_pressure;
    int max_iters;          /* incompressibilityMaxIterationCount */
    double fluid_density;
    double residual_tol;
    int tol_mode;           /* fsim_tol_mode */
    double particle_r;
    int precision;          /* fsim_precision */
    int warm_start;         /* fsim_warm_start */
    int track_ids;          /* keep a stable id per particle (fsim_get_particles in id order) */
    int timing;             /* record per-stage CUDA-event times into fsim_step_stats */
    int precond;            /* fsim_precond (FSIM_PREC_FP64 always uses FSIM_PRECOND_RBIC) */
    int mg_sweeps;          /* multigrid smoothing sweeps before and after the coarse correction on
                               the finest level (0: 1 on grids of 2^23 cells or more, else 2) */
    int mg_coarse_sweeps;   /* the same on level 1 and other levels run as separate kernels (0: 4 on
                               level 1, 6 below it) */
    int mg_cluster_sweeps;  /* the same on the small levels run by one thread-block cluster (0: 8 on
                               the cluster-wide levels, 6 on those one CTA runs alone) */
    int grid_solver;        /* fsim_grid_solver: SimulationConfig::gridSolverType */
    int learned_backoff;    /* FSIM_WARM_LEARNED: after a rejected network guess skip the network on
                               the next 1, 2, 4 ... 64 solves (previous pressure instead); 0: judge
                               the network on every solve */
    int refine_digits;      /* FSIM_PREC_MIXED: fold the FP32 correction into the FP64 pressure and
                               restart from the true FP64 residual each time the residual norm fell
                               10^refine_digits (0: 3) */
    int mg_boundary_sweeps; /* extra red-black sweeps on the finest level's free-surface band (quads
                               within one cell of a fluid cell next to air), after the pre-smoothing
                               and, in reverse order, before the post-smoothing (0: 3 on grids of
                               2^23 cells or more, else none; -1: none; at most 8) */
    int deterministic;      /* 1: bit-reproducible steps (same inputs, same bits on every run):
                               P2G adds into its shared accumulators in one fixed order (one warp
                               per accumulator, smaller tiles; P2G about 1.3x slower).  Every other
                               stage is reproducible in either mode. */
} fsim_params;

/* Obstacle (obstacles.hpp:7-65), speed set by the caller as (pos-prevPos)/dt. */
typedef struct fsim_obstacle {
    int type; /* fsim_obstacle_type */
    double pos[3];
    double prev_pos[3];
    double speed[3];
    double r;       /* spheres, sources, sinks, disc sources */
    double size[3]; /* boxes and box sinks */
    double spawn_rate;  /* sources: particles per second */
    double spawn_speed; /* sources: speed along the normal; disc sources: v_y */
    double last_spawn_fraction;
} fsim_obstacle;

/* SimulationManager::ParticleGfxData (simulationManager.h:74-78). */
typedef struct fsim_particle_gfx {
    float pos[3];
    float v;       /* |velocity| */
    float density; /* trilinear avgPNum at the particle */
} fsim_particle_gfx;

/* Per-step statistics.  stage_ms follows the reference's getStepDuration keys
 * (simulator.cpp:33-40), measured by CUDA events when fsim_params.timing != 0. */
typedef struct fsim_step_stats {
    int pcg_iterations;  /* "Incompressibility it count" */
    int converged;
    int num_particles;
    int num_fluid_cells;
    double residual_max;  /* true residual after the solve, max norm */
    double residual_rel;  /* true residual after the solve, ||r||/||b|| */
    double rhs_norm;
    int guess_used;       /* FSIM_WARM_* actually used */
    int reliable_updates;
    float ms_simulate_particles;  /* "SimulateParticles": spawn + advect + push-out */
    float ms_push_apart;          /* "PushParticlesApart" */
    float ms_push_out;            /* "PushParticlesOutOfObstacles" (fused into advect: 0) */
    float ms_p2g;                 /* "P2GTransfer": sort + P2G + marking */
    float ms_prep;                /* "IncompressibilityPrep": obstacles, walls, v2 */
    float ms_solve;               /* "Incompressibility" */
    float ms_extrapolate;         /* "VelocityExtrapolation" */
    float ms_g2p;                 /* "G2PTransfer" */
    float ms_total;
    float ms_p2g_kernel;          /* the P2G tile kernel alone */
    float ms_g2p_kernel;          /* the G2P tile kernel alone */
    float ms_pcg_setup;           /* solve setup: codes, rhs, bricks, first residual */
    int kernel_launches;          /* CUDA kernels this call launched */
    int num_active_bricks;        /* pressure-solve bricks holding fluid */
    float ms_guess;               /* FSIM_WARM_LEARNED: network inference + residual judgement */
    int reserved[2];
} fsim_step_stats;

typedef struct fsim_ctx fsim_ctx;

/* ---- lifecycle --------------------------------------------------------- */

/* Create a context on the current CUDA device.  Replaces the construction in
 * SimulationManager::SimulationManager (simulationManager.cpp:10-29):
 * BridsonSolverGrid + HashedParticles + Simulator. */
int fsim_create(const fsim_grid_desc *grid, const fsim_params *params, fsim_ctx **out);
int fsim_destroy(fsim_ctx *ctx);
/* Replaces the per-step parameter copy in SimulationManager::simulationThreadWorker
 * (simulationManager.cpp:184-199). */
int fsim_set_params(fsim_ctx *ctx, const fsim_params *params);
int fsim_get_params(fsim_ctx *ctx, fsim_params *out);
/* gridSize (cells), cellD and dimensions of MacGrid (macGrid.h:168-171). */
int fsim_grid_info(fsim_ctx *ctx, int *n3, double *h3, double *dims3);
const char *fsim_last_error(fsim_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t). */
void *fsim_stream(fsim_ctx *ctx);
int fsim_synchronize(fsim_ctx *ctx);

/* ---- particles (HashedParticles, hashedParticles.h:30-177) -------------- */

/* Replace all particles (HashedParticles ctor / setParticleNum + getParticleAt writes).
 * vel and c may be NULL (zero). */
int fsim_set_particles(fsim_ctx *ctx, const float *pos, const float *vel, const float *c,
                       int64_t n, int where);
/* Append particles (HashedParticles::addParticles, hashedParticles.cpp:153-156). */
int fsim_add_particles(fsim_ctx *ctx, const float *pos, const float *vel, const float *c,
                       int64_t n, int where);
/* Copy particles out (getParticleAt / forEach).  With track_ids the order is by
 * particle id, i.e. the order the reference's vector would have; otherwise the
 * device order.  *n receives the count; cap bounds the copy. */
int fsim_get_particles(fsim_ctx *ctx, float *pos, float *vel, float *c, int64_t cap, int64_t *n,
                       int where);
int fsim_num_particles(fsim_ctx *ctx, int64_t *n);

/* ---- obstacles (Simulator::obstacles, simulator.h:74) ------------------- */
int fsim_set_obstacles(fsim_ctx *ctx, const fsim_obstacle *obs, int n);
/* Read back (sources carry last_spawn_fraction between steps). */
int fsim_get_obstacles(fsim_ctx *ctx, fsim_obstacle *obs, int cap, int *n);

/* ---- stepping ---------------------------------------------------------- */

/* One Simulator::simulate(dt) (simulator.cpp:51-100).  stats may be NULL. */
int fsim_step(fsim_ctx *ctx, double dt, fsim_step_stats *stats);
/* One stage of the step, for stage-by-stage checking against the reference's
 * member functions (fsim_stage enum). */
int fsim_stage(fsim_ctx *ctx, int stage, double dt, fsim_step_stats *stats);

/* ---- grid state (MacGrid::cell / getCellAt, macGrid.h:48-93) ------------ */
int fsim_get_grid(fsim_ctx *ctx, int field, void *out, int where);
/* Overwrite a grid field (FLAGS, AVGPNUM, V*, V2*, PRESSURE). */
int fsim_set_grid(fsim_ctx *ctx, int field, const void *in, int where);

/* ---- renderer hand-off (SimulationManager::getParticleGfxData,
 *      simulationManager.cpp:218-231) ------------------------------------- */
int fsim_fill_gfx(fsim_ctx *ctx, fsim_particle_gfx *out, int64_t cap, int64_t *n, int where);
/* The same hand-off without waiting (simulationThreadWorker's publish overlapped
 * with the following steps): the records are written into a device staging
 * buffer on the context's stream and copied to the host buffer `out` on a
 * separate copy stream; the call returns at once with *n.  Pinned or
 * registered `out` gives DMA-engine speed.  Two hand-offs can be in flight
 * (double-buffered staging); `out` must not be read or reused before
 * fsim_gfx_wait returns. */
int fsim_fill_gfx_async(fsim_ctx *ctx, fsim_particle_gfx *out, int64_t cap, int64_t *n);
/* Blocks until every fsim_fill_gfx_async copy has landed in host memory. */
int fsim_gfx_wait(fsim_ctx *ctx);

/* ---- pressure warm start ----------------------------------------------- */
/* Initial guess for the next solve (FP32, reference cell order); used when
 * params.warm_start == FSIM_WARM_GUESS.  No reference counterpart: the
 * reference always starts PCG from zero (bridsonSolverGrid.cpp:249). */
int fsim_set_pressure_guess(fsim_ctx *ctx, const float *p, int where);

/* ---- pressure-only solve (precision study) ------------------------------ */
/* Solve A p = rhs on the current cell flags, with the given precision and
 * tolerance; rhs/out are FP64 in reference cell order (host).  Used to compare
 * the solver variants on identical inputs. */
int fsim_solve_pressure(fsim_ctx *ctx, const double *rhs, double dt, int precision, int tol_mode,
                        double tol, int max_iters, double *p_out, fsim_step_stats *stats);

/* Pressure solve of the current state (the FSIM_STAGE_SOLVE stage,
 * BridsonSolverGrid::solveIncompressibility, bridsonSolverGrid.cpp:244-293)
 * with an explicit warm start; apply == 0 leaves the velocities untouched, so
 * several warm starts can be timed on one problem (stats.ms_solve covers setup,
 * guess and iterations). */
int fsim_solve_current(fsim_ctx *ctx, double dt, int warm_start, int apply, fsim_step_stats *stats);

/* ---- allocation-free particle-to-grid transfer --------------------------
 * This entry point has no counterpart in the reference.  It is for callers
 * that may not allocate GPU memory when they need a transfer: a render or
 * game loop with a fixed frame budget (a device allocation can synchronise the
 * device and stall the frame), a host application that owns the GPU memory
 * pool and gives plugins only the buffers it chose, or a pipeline recorded
 * once and replayed.  It runs the same cell sort and P2G kernels as
 * FSIM_STAGE_P2G (Simulator::p2gTransfer + markFluidCellsAndCalculateParticleDensities)
 * on buffers the caller owns and calls no cudaMalloc, cudaFree or other
 * allocating routine.
 *
 * Scratch.  Its scratch (cell keys, ranks and the sort permutation per
 * particle, counts and starts per cell) lives in one fixed device array of
 * FSIM_NOALLOC_SCRATCH_BYTES compiled into the library.  Every GPU on which
 * the library's kernels are loaded holds that array until the process exits.
 * All calls share it and it keeps the last call's contents (the call clears the
 * part that must start at zero), so calls whose work overlaps on the GPU --
 * on different streams, or from different host threads -- race and must not
 * be issued.  The first call on a device, made with that device current,
 * looks up the array's device address (cudaGetSymbolAddress).  Under CUDA's
 * default lazy module loading, that first call is also where the library's
 * module is loaded on the device and the array reserved, which is a device
 * allocation in effect and can synchronise the device: make the first call at
 * set-up time, before any frame-budgeted work and before capturing any stream
 * (or set CUDA_MODULE_LOADING=EAGER, which reserves it when the library's
 * module loads).
 *
 * Limits.  n <= FSIM_NOALLOC_MAX_PARTICLES and nx*ny*nz <=
 * FSIM_NOALLOC_MAX_CELLS (each axis checked before the product), else
 * FSIM_E_CAPACITY; non-finite or non-positive dims or resolution, or nz not a
 * multiple of 4, give FSIM_E_INVALID.  Grid geometry follows fsim_grid_desc.
 * Positions must lie inside the grid, [0, dims) on every axis, as the
 * context path's advection leaves them; a particle outside is counted in the
 * nearest edge cell, and its weights there have no meaning.
 *
 * Errors.  A CUDA error already pending on the calling thread when the call
 * starts is returned as FSIM_E_CUDA before anything is launched, and left
 * pending for the caller; after that, FSIM_E_CUDA reports this call's own
 * launch failures.
 *
 * Buffers (all device memory, stream-ordered on `stream`, a cudaStream_t or
 * NULL for the default stream): pos and vel hold 3 planes of n floats
 * (component a at pos + a*n), c holds 9 planes (APIC vector c[a] component b
 * at c + (3a+b)*n; may be NULL unless transfer == FSIM_APIC).  Outputs are
 * nx*ny*nz values in the reference cell order: face velocities vx/vy/vz,
 * cell types in flags (WATER where a particle is, AIR elsewhere) and avgPNum. */
#define FSIM_NOALLOC_MAX_PARTICLES (1 << 20)
#define FSIM_NOALLOC_MAX_CELLS (1 << 20)
#define FSIM_NOALLOC_SCRATCH_BYTES 20973312
int fsim_p2g_noalloc(const fsim_grid_desc *grid, int transfer, const float *pos, const float *vel,
                     const float *c, int64_t n, float *vx, float *vy, float *vz, uint8_t *flags,
                     float *avg, void *stream);

/* ---- learned pressure warm start -----------------------------------------
 * No counterpart in the reference (its PCG starts from zero,
 * bridsonSolverGrid.cpp:249).  A 3D U-Net (levels of 16, 32, 64, 64 channels,
 * two 3x3x3 conv + ReLU per level, 2x2x2 stride-2 down-convolutions, trilinear
 * up-sampling with skip concatenation, 1x1x1 head) maps the solver's scaled
 * right-hand side and cell types to a pressure guess.  BF16 weights and
 * activations, FP32 accumulation on the tensor cores, FP32 master parameters
 * trained with Adam.  The guess only seeds PCG: with params.warm_start ==
 * FSIM_WARM_LEARNED (the network's pressure) or FSIM_WARM_LEARNED_RESIDUAL (the
 * previous step's pressure plus the network's answer to the residual that
 * pressure leaves) the solver compares the guess's residual with that of the
 * previous step's pressure, starts from the better one and iterates to the
 * same tolerance.
 *
 * Network input: [n][d][h][w][4] FP32 = (rhs / rms(rhs over fluid cells),
 * fluid, solid, air); output [n][d][h][w] FP32 = pressure / rms(rhs), both in
 * the solver's integer-stencil units (A = 7-point Laplacian with unit
 * off-diagonals).  d, h, w are multiples of 8; voxel (d, h, w) is cell
 * (x, y, z).  Parameters are one flat FP32 array (layer by layer: weights
 * [tap][cout][cin], bias [cout]; head weight [16], bias [1]). */
typedef struct fsim_net fsim_net;
int fsim_net_create(uint64_t seed, float out_scale, fsim_net **out);
int fsim_net_destroy(fsim_net *net);
const char *fsim_net_last_error(const fsim_net *net);
int64_t fsim_net_num_params(const fsim_net *net);
/* what: 0 parameters, 1 accumulated gradient */
int fsim_net_get_params(fsim_net *net, float *dst, int what, int where);
int fsim_net_set_params(fsim_net *net, const float *src, int where);
/* Forward pass; train != 0 keeps what fsim_net_backward needs.  out may be NULL. */
int fsim_net_forward(fsim_net *net, int n, int d, int h, int w, const float *in, float *out, int train,
                     int where);
/* Backward pass after a training forward pass (batch n <= 64); adds to the
 * gradient.  target [n][d][h][w] FP32 is the plain solver's solution, mask
 * (uint8) marks the fluid cells.  Per sample, with e = prediction - target on
 * fluid cells, A the solver's 7-point operator of the input's cell types and
 * b the scaled rhs (input channel 0; A target = b, so A e is the residual the
 * guess leaves in PCG), the loss is the mean over the batch of
 *   ||A e|| / ||b|| + l2_weight * ||e|| / ||target||
 * (relative residual plus relative L2 error to the solver's pressure). */
int fsim_net_backward(fsim_net *net, const float *target, const uint8_t *mask, float *loss, int where);
/* l2_weight of the loss (default 0.1). */
int fsim_net_set_loss(fsim_net *net, float l2_weight);
/* One Adam step on a batch drawn from a training pool resident in device
 * memory, without synchronising the host: sample b of the batch is pool
 * sample idx[b] (device int array of `batch` entries, batch <= 64).  Pool
 * arrays hold [samples][d][h][w]: types (uint8: 0 fluid unknown, 1 air,
 * 2 solid), rhs and target (FP32, scaled as for fsim_net_forward / backward).
 * loss_out (device float, may be NULL) receives the batch loss when the step
 * has run; errors of the tensor-core kernels surface at fsim_net_synchronize. */
int fsim_net_train_batch(fsim_net *net, int d, int h, int w, const uint8_t *types, const float *rhs,
                         const float *target, const int *idx, int batch, float lr, float *loss_out);
int fsim_net_zero_grad(fsim_net *net);
/* Adam (beta 0.9 / 0.999, eps 1e-8) on the accumulated gradient, which it clears. */
int fsim_net_adam(fsim_net *net, float lr);
/* forward + backward + Adam on one batch */
int fsim_net_train_step(fsim_net *net, int n, int d, int h, int w, const float *in, const float *target,
                        const uint8_t *mask, float lr, float *loss, int where);
int fsim_net_synchronize(fsim_net *net);
/* One convolution of the network's kernels on FP32 arrays (rounded to BF16
 * inside), for checks: mode 0 forward y = conv(x, w) ([vox][cout]), mode 1
 * input gradient of g ([vox][cin]), mode 2 weight gradient sum x (x) g
 * ([taps][cout][cin]).  taps 27 (3x3x3, padding 1) or 1; cin, cout multiples
 * of 16 (mode 2: cout <= 64). */
int fsim_net_conv(int taps, int mode, int n, int d, int h, int w, int cin, int cout, const float *x,
                  const float *wgt, const float *g, float *out, int where);
/* Attach (or detach with NULL) the network used by FSIM_WARM_LEARNED.  The
 * context does not own it. */
int fsim_set_net(fsim_ctx *ctx, fsim_net *net);

#ifdef __cplusplus
}
#endif

#endif /* FSIM_H */
