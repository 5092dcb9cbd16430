/*
 * oracle_api.h -- C interface shared by the two CPU oracles (test infrastructure
 * only; nothing in the product links against it).
 *
 *   oracle/_ref/libfsim_ref.so   the reference's own Simulator sources
 *                                (the .cpp files under src/Simulator/simulator) compiled
 *                                against oracle/glmshim and driven by
 *                                oracle/ref_harness.cpp.  Built only where the
 *                                reference sources are present.
 *   oracle/liboracle.so          oracle/fsim_oracle.c: a plain-C FP64
 *                                restatement of the same per-step algorithm,
 *                                pinned against the reference library through
 *                                the golden fixtures under tests/golden/.
 *
 * Both export exactly these symbols, so tests drive either one the same way.
 * All arrays are FP64 AoS per particle (pos[3*n], vel[3*n], c[9*n]; c row a =
 * the APIC vector c[a] of the reference's Particle, particle.h:8-12) and
 * x-major cell order index = (x*ny + y)*nz + z, like MacGrid::cell
 * (macGrid.h:91-93).
 */
#ifndef FSIM_ORACLE_API_H
#define FSIM_ORACLE_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum oracle_transfer { ORACLE_PIC = 0, ORACLE_FLIP = 1, ORACLE_APIC = 2 };

/* Cell types, same order as MacGridCell::CellType (macGridCell.h:29-31). */
enum oracle_cell { ORACLE_WATER = 0, ORACLE_AIR = 1, ORACLE_SOLID = 2 };

enum oracle_obstacle_type {
    ORACLE_OBS_SPHERE = 0, /* SphericalObstacle (obstacles.hpp:36-44) */
    ORACLE_OBS_BOX = 1,    /* RectengularObstacle (obstacles.hpp:26-34) */
    ORACLE_OBS_SOURCE = 2, /* SphericalParticleSource (obstacles.hpp:46-57) */
    ORACLE_OBS_SINK = 3,   /* SphericalParticleSink (obstacles.hpp:59-65) */
    /* extensions of the 256^3 benchmark workload (no reference counterpart;
     * the reference library ignores them) */
    ORACLE_OBS_DISC_SOURCE = 4, /* horizontal disc: 8 jittered particles per covered cell per step */
    ORACLE_OBS_BOX_SINK = 5     /* axis-aligned box deleting particles */
};

typedef struct oracle_params {
    double resolution;          /* cells per unit length (MacGrid ctor, macGrid.cpp:9-13) */
    double dims[3];             /* target dimensions */
    int two_d;                  /* 2D mode (z is 3 cells) */
    double particle_r;          /* HashedParticles radius */
    int transfer;               /* oracle_transfer */
    float flip_ratio;           /* SimulatorConfig::flipRatio (float, simulator.h:32) */
    float gravity;              /* SimulatorConfig::gravity (float, simulator.h:33) */
    int gravity_enabled;
    int push_apart_enabled;
    int spawning_enabled;
    int despawning_enabled;
    int stop_particles;
    int top_solid;              /* MacGrid::isTopOfContainerSolid */
    int pressure_enabled;       /* MacGrid::pressureEnabled */
    int max_iters;              /* MacGrid::incompressibilityMaxIterationCount */
    double pressure_k;
    double average_pressure;
    double fluid_density;
    double residual_tol;        /* MacGrid::residualTolerance (absolute max-norm) */
    int grid_solver;            /* 0 BridsonSolverGrid (PCG), 1 BasicMacGrid (SOR) --
                                   SimulationConfig::gridSolverType (simulationManager.cpp:16-19) */
} oracle_params;

typedef struct oracle_obstacle {
    int type;                   /* oracle_obstacle_type */
    double pos[3];
    double prev_pos[3];
    double speed[3];
    double r;                   /* spheres, sources, sinks */
    double size[3];             /* boxes */
    double spawn_rate;          /* sources: particles per second */
    double spawn_speed;         /* sources */
    double last_spawn_fraction; /* sources (carried between steps) */
} oracle_obstacle;

/* Stage ids, in the order Simulator::simulate runs them (simulator.cpp:51-100). */
enum oracle_stage {
    ORACLE_STAGE_SPAWN = 0,
    ORACLE_STAGE_ADVECT = 1,
    ORACLE_STAGE_PUSH_APART = 2,
    ORACLE_STAGE_PUSH_OUT = 3,
    ORACLE_STAGE_STOP = 4,
    ORACLE_STAGE_P2G = 5,          /* resetGridValues + p2gTransfer */
    ORACLE_STAGE_MARK = 6,
    ORACLE_STAGE_OBSTACLES = 7,
    ORACLE_STAGE_WALLS = 8,
    ORACLE_STAGE_POST_P2G = 9,     /* v2 = v (+gravity), fluid list */
    ORACLE_STAGE_SOLVE = 10,
    ORACLE_STAGE_EXTRAPOLATE = 11,
    ORACLE_STAGE_G2P = 12
};

/* Grid fields for oracle_get_grid / oracle_set_grid. */
enum oracle_field {
    ORACLE_F_FLAGS = 0,    /* uint8 cell type */
    ORACLE_F_AVGPNUM = 1,  /* double */
    ORACLE_F_VX = 2, ORACLE_F_VY = 3, ORACLE_F_VZ = 4,       /* face v (double) */
    ORACLE_F_V2X = 5, ORACLE_F_V2Y = 6, ORACLE_F_V2Z = 7,    /* face v2 (double) */
    ORACLE_F_PRESSURE = 8, /* double, last solve, 0 outside fluid */
    ORACLE_F_WX = 9, ORACLE_F_WY = 10, ORACLE_F_WZ = 11,     /* P2G weight sums */
    ORACLE_F_FLUID_ID = 12 /* int32, -1 outside fluid */
};

void *oracle_create(const oracle_params *p, int n, const double *pos, const double *vel,
                    const double *c);
void oracle_destroy(void *h);
void oracle_set_threads(int n);
void oracle_grid_size(void *h, int *n3);
void oracle_cell_size(void *h, double *h3);
int oracle_num_particles(void *h);
void oracle_get_particles(void *h, double *pos, double *vel, double *c);
void oracle_set_particles(void *h, int n, const double *pos, const double *vel, const double *c);
void oracle_set_params(void *h, const oracle_params *p);
void oracle_set_obstacles(void *h, int n, const oracle_obstacle *obs);
int oracle_get_obstacles(void *h, int cap, oracle_obstacle *obs);
/* One full Simulator::simulate(dt).  Returns the PCG iteration count. */
int oracle_step(void *h, double dt);
/* One stage; returns the PCG iteration count for ORACLE_STAGE_SOLVE, else 0. */
int oracle_stage(void *h, int stage, double dt);
void oracle_get_grid(void *h, int field, void *out);
/* Overwrite a grid field; ORACLE_F_FLAGS also rebuilds the fluid-cell list
 * (lexicographic over interior cells, like MacGrid::postP2GUpdate). */
void oracle_set_grid(void *h, int field, const void *in);
int oracle_fluid_count(void *h);
int oracle_last_iterations(void *h);

#ifdef __cplusplus
}
#endif

#endif
