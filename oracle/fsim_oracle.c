/*
 * fsim_oracle.c -- CPU oracle: an FP64 plain-C restatement of the reference's
 * per-step simulation path (dkiovics/fluid_simulator, src/Simulator/simulator).
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA path's tests and __graft_entry__.smoke
 * compare against it, and bench.py times it as the CPU baseline; the product
 * never links or calls it.  It follows the reference operation by operation
 * (same expression order, separately rounded FP64 multiplies and adds), so with
 * one thread it reproduces the reference bit for bit; tests/test_oracle_golden.py
 * pins that against fixtures generated from the reference's own sources.
 *
 * Layout: particles AoS FP64 (pos, v, c[3]); grid SoA FP64 with the reference's
 * x-major cell order (macGrid.h:91-93).  OpenMP parallelises the same loops the
 * reference parallelises (P2G/density scatter with atomics); run with one thread
 * for bit-exact parity.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_api.h"

/* M_PI of the C library headers (not visible under -std=c11). */
#define FSIM_PI 3.14159265358979323846

typedef struct {
    double x, y, z;
} d3;

static inline double d3_get(const d3 *v, int a) { return a == 0 ? v->x : (a == 1 ? v->y : v->z); }
static inline void d3_set(d3 *v, int a, double s) {
    if (a == 0) v->x = s; else if (a == 1) v->y = s; else v->z = s;
}
static inline double d3_dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

typedef struct {
    d3 pos, v, c[3];
} particle;

typedef struct {
    oracle_params p;
    int nx, ny, nz, ncell, yz;
    d3 cd, cdi, dims;
    /* particles */
    int n, cap;
    particle *pt;
    /* grid */
    uint8_t *type;
    double *v[3], *v2[3], *w[3], *avg, *pressure;
    int32_t *id;
    int nfluid;
    int32_t *fluid; /* linear cell index of each fluid cell, lexicographic */
    int last_its;
    /* obstacles */
    int nobs;
    oracle_obstacle *obs;
} sim;

static inline int cidx(const sim *s, int x, int y, int z) { return x * s->yz + y * s->nz + z; }

/* ---------------------------------------------------------------- geometry */

/* Face centre of axis a of cell (x,y,z) (macGrid.cpp:25-27). */
static inline d3 face_pos(const sim *s, int a, int x, int y, int z) {
    d3 r;
    r.x = (a == 0) ? (double)(x + 1) * s->cd.x : (x + 0.5) * s->cd.x;
    r.y = (a == 1) ? (double)(y + 1) * s->cd.y : (y + 0.5) * s->cd.y;
    r.z = (a == 2) ? (double)(z + 1) * s->cd.z : (z + 0.5) * s->cd.z;
    return r;
}

/* Cell centre (macGrid.cpp:28). */
static inline d3 cell_pos(const sim *s, int x, int y, int z) {
    d3 r = {(x + 0.5) * s->cd.x, (y + 0.5) * s->cd.y, (z + 0.5) * s->cd.z};
    return r;
}

/* trilinearInterpoll (util/interpolation.h:7-18). */
static inline double tri_w(d3 center, d3 pos, d3 inv) {
    double vx = (pos.x - center.x) * inv.x, vy = (pos.y - center.y) * inv.y,
           vz = (pos.z - center.z) * inv.z;
    double x = 1.0 - fabs(vx), y = 1.0 - fabs(vy), z = 1.0 - fabs(vz);
    return x * y * z;
}

/* trilinearInterpollGradient (util/interpolation.h:21-35). */
static inline d3 tri_grad(d3 center, d3 pos, d3 inv) {
    double vx = (pos.x - center.x) * inv.x, vy = (pos.y - center.y) * inv.y,
           vz = (pos.z - center.z) * inv.z;
    double xa = 1.0 - fabs(vx), ya = 1.0 - fabs(vy), za = 1.0 - fabs(vz);
    double xs = vx > 0.0 ? -1.0 : 1.0, ys = vy > 0.0 ? -1.0 : 1.0, zs = vz > 0.0 ? -1.0 : 1.0;
    d3 g = {xs * ya * za * inv.x, ys * xa * za * inv.y, zs * xa * ya * inv.z};
    return g;
}

/* Stencil offsets in the order of getFacesAround / getCellsAround
 * (macGrid.cpp:150-201). */
static const int OFF[8][3] = {{1, 1, 1}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0},
                              {1, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 0, 0}};

/* Lower stencil corner for face axis a (macGrid.cpp:143-148): trunc of
 * pos/h - offset_a, minus one along a. */
static inline void face_base(const sim *s, d3 pos, int a, int *b) {
    double gx = pos.x * s->cdi.x - (a == 0 ? 0.0 : 0.5);
    double gy = pos.y * s->cdi.y - (a == 1 ? 0.0 : 0.5);
    double gz = pos.z * s->cdi.z - (a == 2 ? 0.0 : 0.5);
    b[0] = (int)gx;
    b[1] = (int)gy;
    b[2] = (int)gz;
    b[a] -= 1;
}

/* ------------------------------------------------------------- lifecycle */

static void grid_alloc(sim *s) {
    const oracle_params *p = &s->p;
    double res = (double)(float)p->resolution; /* BridsonSolverGrid takes a float */
    s->cd.x = 1 / res;
    s->cd.y = 1 / res;
    s->cd.z = p->two_d ? p->dims[2] / 3 : 1 / res;
    s->cdi.x = 1.0 / s->cd.x;
    s->cdi.y = 1.0 / s->cd.y;
    s->cdi.z = 1.0 / s->cd.z;
    s->nx = (int)(p->dims[0] / s->cd.x);
    s->ny = (int)(p->dims[1] / s->cd.y);
    s->nz = p->two_d ? 3 : (int)(p->dims[2] / s->cd.z);
    s->dims.x = s->nx * s->cd.x;
    s->dims.y = s->ny * s->cd.y;
    s->dims.z = p->two_d ? p->dims[2] : s->nz * s->cd.z;
    s->yz = s->ny * s->nz;
    s->ncell = s->nx * s->ny * s->nz;
    size_t n = (size_t)s->ncell;
    s->type = (uint8_t *)calloc(n, 1);
    for (int a = 0; a < 3; a++) {
        s->v[a] = (double *)calloc(n, sizeof(double));
        s->v2[a] = (double *)calloc(n, sizeof(double));
        s->w[a] = (double *)calloc(n, sizeof(double));
    }
    s->avg = (double *)calloc(n, sizeof(double));
    s->pressure = (double *)calloc(n, sizeof(double));
    s->id = (int32_t *)calloc(n, sizeof(int32_t));
    s->fluid = (int32_t *)malloc(n * sizeof(int32_t));
    for (size_t i = 0; i < n; i++) s->type[i] = ORACLE_AIR;
}

static void walls(sim *s);

static void particles_resize(sim *s, int n) {
    if (n > s->cap) {
        int cap = s->cap ? s->cap : 1024;
        while (cap < n) cap *= 2;
        s->pt = (particle *)realloc(s->pt, (size_t)cap * sizeof(particle));
        s->cap = cap;
    }
    s->n = n;
}

static void write_particles(sim *s, int n, const double *pos, const double *vel, const double *c) {
    particles_resize(s, n);
    for (int i = 0; i < n; i++) {
        particle *q = &s->pt[i];
        q->pos.x = pos[3 * i]; q->pos.y = pos[3 * i + 1]; q->pos.z = pos[3 * i + 2];
        q->v.x = vel ? vel[3 * i] : 0.0;
        q->v.y = vel ? vel[3 * i + 1] : 0.0;
        q->v.z = vel ? vel[3 * i + 2] : 0.0;
        for (int a = 0; a < 3; a++) {
            q->c[a].x = c ? c[9 * i + 3 * a] : 0.0;
            q->c[a].y = c ? c[9 * i + 3 * a + 1] : 0.0;
            q->c[a].z = c ? c[9 * i + 3 * a + 2] : 0.0;
        }
    }
}

void *oracle_create(const oracle_params *p, int n, const double *pos, const double *vel,
                    const double *c) {
    sim *s = (sim *)calloc(1, sizeof(sim));
    s->p = *p;
    grid_alloc(s);
    walls(s); /* the MacGrid ctor marks the walls (macGrid.cpp:16) */
    write_particles(s, n, pos, vel, c);
    return s;
}

void oracle_destroy(void *h) {
    sim *s = (sim *)h;
    if (!s) return;
    free(s->type);
    for (int a = 0; a < 3; a++) { free(s->v[a]); free(s->v2[a]); free(s->w[a]); }
    free(s->avg); free(s->pressure); free(s->id); free(s->fluid); free(s->pt); free(s->obs);
    free(s);
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void oracle_grid_size(void *h, int *n3) {
    sim *s = (sim *)h;
    n3[0] = s->nx; n3[1] = s->ny; n3[2] = s->nz;
}

void oracle_cell_size(void *h, double *h3) {
    sim *s = (sim *)h;
    h3[0] = s->cd.x; h3[1] = s->cd.y; h3[2] = s->cd.z;
}

int oracle_num_particles(void *h) { return ((sim *)h)->n; }

void oracle_get_particles(void *h, double *pos, double *vel, double *c) {
    sim *s = (sim *)h;
    for (int i = 0; i < s->n; i++) {
        const particle *q = &s->pt[i];
        for (int a = 0; a < 3; a++) {
            if (pos) pos[3 * i + a] = d3_get(&q->pos, a);
            if (vel) vel[3 * i + a] = d3_get(&q->v, a);
            if (c) {
                c[9 * i + 3 * a] = q->c[a].x;
                c[9 * i + 3 * a + 1] = q->c[a].y;
                c[9 * i + 3 * a + 2] = q->c[a].z;
            }
        }
    }
}

void oracle_set_particles(void *h, int n, const double *pos, const double *vel, const double *c) {
    write_particles((sim *)h, n, pos, vel, c);
}

void oracle_set_params(void *h, const oracle_params *p) {
    sim *s = (sim *)h;
    /* grid geometry is fixed at creation; the remaining fields are live */
    oracle_params keep = s->p;
    s->p = *p;
    s->p.resolution = keep.resolution;
    memcpy(s->p.dims, keep.dims, sizeof(keep.dims));
    s->p.two_d = keep.two_d;
}

void oracle_set_obstacles(void *h, int n, const oracle_obstacle *obs) {
    sim *s = (sim *)h;
    free(s->obs);
    s->obs = NULL;
    s->nobs = n;
    if (n > 0) {
        s->obs = (oracle_obstacle *)malloc((size_t)n * sizeof(oracle_obstacle));
        memcpy(s->obs, obs, (size_t)n * sizeof(oracle_obstacle));
    }
}

int oracle_get_obstacles(void *h, int cap, oracle_obstacle *obs) {
    sim *s = (sim *)h;
    for (int i = 0; i < s->nobs && i < cap; i++) obs[i] = s->obs[i];
    return s->nobs;
}

static inline int is_spherical(int t) {
    return t == ORACLE_OBS_SPHERE || t == ORACLE_OBS_SOURCE || t == ORACLE_OBS_SINK;
}

static inline d3 obs_pos(const oracle_obstacle *o) { d3 r = {o->pos[0], o->pos[1], o->pos[2]}; return r; }
static inline d3 obs_speed(const oracle_obstacle *o) { d3 r = {o->speed[0], o->speed[1], o->speed[2]}; return r; }

/* ------------------------------------------------------------ spawn (a6) */

/* Simulator::spawnParticles (simulator.cpp:106-125); util::getDoubleInRange
 * (util/random.h:23-25) on the C library's rand(). */
static double rand_in(double lo, double hi) { return lo + (hi - lo) * ((double)rand() / RAND_MAX); }

/* Disc source (extension): 8 particles per covered cell of the cell row at
 * pos.y, one per 2x2x2 sub-cell with +-0.5 sub-cell jitter, velocity (0, speed, 0). */
static void spawn_disc(sim *s, const oracle_obstacle *o) {
    const double h = s->cd.x;
    const int cy = (int)(o->pos[1] * s->cdi.y);
    if (cy < 1 || cy >= s->ny - 1) return;
    const double cx = o->pos[0] * s->cdi.x, cz = o->pos[2] * s->cdi.z, r = o->r * s->cdi.x;
    for (int x = 1; x < s->nx - 1; x++)
        for (int z = 1; z < s->nz - 1; z++) {
            const double dx = x + 0.5 - cx, dz = z + 0.5 - cz;
            if (dx * dx + dz * dz > r * r) continue;
            for (int q = 0; q < 8; q++) {
                const double sub[3] = {(q & 4) ? 0.75 : 0.25, (q & 2) ? 0.75 : 0.25, (q & 1) ? 0.75 : 0.25};
                const double base[3] = {(double)x, (double)cy, (double)z};
                int idx = s->n;
                particles_resize(s, s->n + 1);
                particle *p = &s->pt[idx];
                double c[3];
                for (int a = 0; a < 3; a++) c[a] = (base[a] + sub[a] + (rand_in(0.0, 1.0) - 0.5) * 0.5 * 0.999) * h;
                p->pos.x = c[0]; p->pos.y = c[1]; p->pos.z = c[2];
                p->v.x = 0.0; p->v.y = o->spawn_speed; p->v.z = 0.0;
                memset(p->c, 0, sizeof(p->c));
            }
        }
}

static void stage_spawn(sim *s, double dt) {
    const double pr = s->p.particle_r;
    for (int k = 0; k < s->nobs; k++) {
        oracle_obstacle *o = &s->obs[k];
        if (o->type == ORACLE_OBS_DISC_SOURCE) { spawn_disc(s, o); continue; }
        if (o->type != ORACLE_OBS_SOURCE) continue;
        double r = o->r + pr;
        double numd = o->spawn_rate * dt + o->last_spawn_fraction;
        int num = (int)numd;
        o->last_spawn_fraction = numd - num;
        for (int i = 0; i < num; i++) {
            double theta = rand_in(0.0, 2.0 * FSIM_PI);
            double phi = rand_in(0.0, FSIM_PI);
            d3 nrm = {r * sin(phi) * cos(theta), r * sin(phi) * sin(theta), r * cos(phi)};
            double inv = 1.0 / sqrt(d3_dot(nrm, nrm));
            int idx = s->n;
            particles_resize(s, s->n + 1);
            particle *q = &s->pt[idx];
            q->pos.x = o->pos[0] + nrm.x; q->pos.y = o->pos[1] + nrm.y; q->pos.z = o->pos[2] + nrm.z;
            q->v.x = o->spawn_speed * (nrm.x * inv);
            q->v.y = o->spawn_speed * (nrm.y * inv);
            q->v.z = o->spawn_speed * (nrm.z * inv);
            memset(q->c, 0, sizeof(q->c));
        }
    }
}

/* ----------------------------------------------------------- advect (a5) */

/* isParticleInRectangle (simulator.cpp:127-132). */
static inline int in_rect(d3 p, double pr, d3 rp, const double *size) {
    return (fabs(p.x - rp.x) < size[0] * 0.5 + pr) && (fabs(p.y - rp.y) < size[1] * 0.5 + pr) &&
           (fabs(p.z - rp.z) < size[2] * 0.5 + pr);
}

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Simulator::advectParticles (simulator.cpp:134-251). */
static void stage_advect(sim *s, double dt) {
    const double wallRest = 0.3, sphereRest = 1.0, rectRest = 0.2;
    const double pr = s->p.particle_r;
    d3 lo = {s->cd.x + pr * 1.01, s->cd.y + pr * 1.01, s->cd.z + (s->p.two_d ? 0.0 : pr) * 1.01};
    d3 hi = {s->dims.x - lo.x, s->dims.y - lo.y, s->dims.z - lo.z};
    int *remove = (int *)malloc((size_t)(s->n > 0 ? s->n : 1) * sizeof(int));
    int nremove = 0;
    const int despawn = s->p.despawning_enabled;

#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < s->n; idx++) {
        particle *q = &s->pt[idx];
        double t = 0;
        int run = 0;
        const int maxRun = 200;
        while (run < maxRun) {
            run++;
            double minT = 1e6;
            int minAxis = 0;
            for (int a = 0; a < 3; a++) {
                double comp = d3_get(&q->v, a), tmp = 1e6;
                if (comp > 1e-6)
                    tmp = (d3_get(&hi, a) - d3_get(&q->pos, a)) / comp;
                else if (comp < -1e-6)
                    tmp = (d3_get(&q->pos, a) - d3_get(&lo, a)) / -comp;
                if (tmp < minT) { minT = tmp; minAxis = a; }
            }
            if (minT <= (dt - t)) {
                q->pos.x = q->pos.x + q->v.x * minT * 0.999;
                q->pos.y = q->pos.y + q->v.y * minT * 0.999;
                q->pos.z = q->pos.z + q->v.z * minT * 0.999;
                d3_set(&q->v, minAxis, d3_get(&q->v, minAxis) * -wallRest);
                t += 0.999 * minT;
                continue;
            }
            int collision = 0;
            double rem = dt - t;
            q->pos.x = q->pos.x + q->v.x * rem;
            q->pos.y = q->pos.y + q->v.y * rem;
            q->pos.z = q->pos.z + q->v.z * rem;
            for (int k = 0; k < s->nobs; k++) {
                const oracle_obstacle *o = &s->obs[k];
                d3 op = obs_pos(o), os = obs_speed(o);
                if (o->type == ORACLE_OBS_BOX_SINK) {
                    if (despawn && fabs(q->pos.x - op.x) < o->size[0] * 0.5 &&
                        fabs(q->pos.y - op.y) < o->size[1] * 0.5 && fabs(q->pos.z - op.z) < o->size[2] * 0.5) {
#pragma omp critical(fsim_oracle_remove)
                        remove[nremove++] = idx;
                        collision = 0;
                        break;
                    }
                    continue;
                }
                if (is_spherical(o->type)) {
                    int isSink = o->type == ORACLE_OBS_SINK;
                    double r = o->r + pr;
                    d3 dd = {op.x - q->pos.x, op.y - q->pos.y, op.z - q->pos.z};
                    double d = sqrt(d3_dot(dd, dd)) - r;
                    if (d < 0) {
                        if (isSink && despawn) {
#pragma omp critical(fsim_oracle_remove)
                            remove[nremove++] = idx;
                            collision = 0;
                            break;
                        }
                        double bt = 0;
                        for (;;) {
                            d3 e = {(q->pos.x - q->v.x * bt) - (op.x - os.x * bt),
                                    (q->pos.y - q->v.y * bt) - (op.y - os.y * bt),
                                    (q->pos.z - q->v.z * bt) - (op.z - os.z * bt)};
                            if (!(sqrt(d3_dot(e, e)) < r && bt < t + (double)0.001f)) break;
                            bt += 0.0002;
                        }
                        if (bt > dt - t) continue;
                        bt += 0.0002;
                        q->pos.x -= bt * q->v.x;
                        q->pos.y -= bt * q->v.y;
                        q->pos.z -= bt * q->v.z;
                        d3 ptmp = {op.x - os.x * bt, op.y - os.y * bt, op.z - os.z * bt};
                        d3 nd = {q->pos.x - ptmp.x, q->pos.y - ptmp.y, q->pos.z - ptmp.z};
                        double inv = 1.0 / sqrt(d3_dot(nd, nd));
                        d3 nrm = {nd.x * inv, nd.y * inv, nd.z * inv};
                        d3 rv = {q->v.x - os.x, q->v.y - os.y, q->v.z - os.z};
                        double semi = -d3_dot(nrm, rv);
                        if (semi <= 0.0f) continue;
                        d3 mir = {-rv.x / semi, -rv.y / semi, -rv.z / semi};
                        q->v.x = (nrm.x - mir.x) * 2.0 + mir.x;
                        q->v.y = (nrm.y - mir.y) * 2.0 + mir.y;
                        q->v.z = (nrm.z - mir.z) * 2.0 + mir.z;
                        double f = semi * sphereRest;
                        q->v.x *= f; q->v.y *= f; q->v.z *= f;
                        q->v.x += os.x; q->v.y += os.y; q->v.z += os.z;
                        t += (dt - t) - bt;
                        collision = 1;
                        break;
                    }
                }
                if (o->type == ORACLE_OBS_BOX) {
                    if (in_rect(q->pos, pr, op, o->size)) {
                        double bt = 0;
                        for (;;) {
                            d3 pp = {q->pos.x - q->v.x * bt, q->pos.y - q->v.y * bt, q->pos.z - q->v.z * bt};
                            d3 oo = {op.x - os.x * bt, op.y - os.y * bt, op.z - os.z * bt};
                            if (!(in_rect(pp, pr, oo, o->size) && bt < dt - t)) break;
                            bt += 0.0002;
                        }
                        if (bt > dt - t) continue;
                        bt += 0.0002;
                        q->pos.x -= bt * q->v.x;
                        q->pos.y -= bt * q->v.y;
                        q->pos.z -= bt * q->v.z;
                        d3 ptmp = {op.x - os.x * bt, op.y - os.y * bt, op.z - os.z * bt};
                        for (int a = 0; a < 3; a++) {
                            double pa = d3_get(&q->pos, a), ta = d3_get(&ptmp, a);
                            if (pa >= ta + o->size[a] * 0.5 + pr) {
                                d3_set(&q->v, a, -d3_get(&q->v, a) * rectRest + d3_get(&os, a));
                                break;
                            } else if (pa <= ta - o->size[a] * 0.5 - pr) {
                                d3_set(&q->v, a, -d3_get(&q->v, a) * rectRest - d3_get(&os, a));
                                break;
                            }
                        }
                        t += (dt - t) - bt;
                        collision = 1;
                        break;
                    }
                }
            }
            if (!collision) run = maxRun;
        }
        for (int a = 0; a < 3; a++) {
            double v = d3_get(&q->pos, a), l = d3_get(&lo, a), hh = d3_get(&hi, a);
            d3_set(&q->pos, a, v < l ? l : (hh < v ? hh : v));
        }
    }

    /* HashedParticles::removeParticles (hashedParticles.cpp:158-172): stable compaction */
    if (nremove > 0) {
        qsort(remove, (size_t)nremove, sizeof(int), cmp_int);
        int ri = 0;
        for (int p = 0; p < s->n; p++) {
            if (ri < nremove && p == remove[ri]) { ri++; continue; }
            s->pt[p - ri] = s->pt[p];
        }
        s->n -= nremove;
    }
    free(remove);
}

/* -------------------------------------------------------- push out (a7) */

static inline double clampd(double v, double lo, double hi) { return v < lo ? lo : (hi < v ? hi : v); }

/* Simulator::pushParticlesOutOfObstacles (simulator.cpp:253-312);
 * MacGrid::getMinMaxRect (macGrid.h:139-145). */
/* HashedParticles::pushParticlesApart (hashedParticles.cpp:64-107) with the
 * GPU library's deterministic (Jacobi) semantics: from the positions at the
 * start of the pass, every particle moves by the sum over all others within
 * 2r (and at least 1e-4 away) of half the overlap along their separation, then
 * is clamped to [h + 1.01 r, dims - h - 1.01 r].  The reference moves both
 * particles of a pair in place in a racy parallel loop, so it has no single
 * result to restate; for an isolated pair both agree.  O(n) with a cell hash of
 * edge h (neighbours within 2r <= h are in the 27 surrounding cells). */
static void stage_push_apart(sim *s) {
    const int n = s->n;
    if (n <= 0) return;
    const double r = s->p.particle_r, D = 2.0 * r, D2 = D * D;
    const double lo[3] = {s->cd.x + r * 1.01, s->cd.y + r * 1.01, s->cd.z + r * 1.01};
    const double hi[3] = {s->dims.x - lo[0], s->dims.y - lo[1], s->dims.z - lo[2]};
    int *cnt = (int *)calloc((size_t)s->ncell + 1, sizeof(int));
    int *idx = (int *)malloc((size_t)n * sizeof(int));
    int *key = (int *)malloc((size_t)n * sizeof(int));
    for (int i = 0; i < n; i++) {
        int cx = (int)(s->pt[i].pos.x * s->cdi.x), cy = (int)(s->pt[i].pos.y * s->cdi.y),
            cz = (int)(s->pt[i].pos.z * s->cdi.z);
        cx = cx < 0 ? 0 : (cx >= s->nx ? s->nx - 1 : cx);
        cy = cy < 0 ? 0 : (cy >= s->ny ? s->ny - 1 : cy);
        cz = cz < 0 ? 0 : (cz >= s->nz ? s->nz - 1 : cz);
        key[i] = cx * s->yz + cy * s->nz + cz;
        cnt[key[i] + 1]++;
    }
    for (int c = 0; c < s->ncell; c++) cnt[c + 1] += cnt[c];
    int *fill = (int *)malloc((size_t)s->ncell * sizeof(int));
    memcpy(fill, cnt, (size_t)s->ncell * sizeof(int));
    for (int i = 0; i < n; i++) idx[fill[key[i]]++] = i;
    d3 *np = (d3 *)malloc((size_t)n * sizeof(d3));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        const d3 pi = s->pt[i].pos;
        const int c = key[i], cx = c / s->yz, cy = (c / s->nz) % s->ny, cz = c % s->nz;
        double dx = 0.0, dy = 0.0, dz = 0.0;
        for (int x = cx - 1; x <= cx + 1; x++)
            for (int y = cy - 1; y <= cy + 1; y++)
                for (int z = cz - 1; z <= cz + 1; z++) {
                    if (x < 0 || y < 0 || z < 0 || x >= s->nx || y >= s->ny || z >= s->nz) continue;
                    const int cc = x * s->yz + y * s->nz + z;
                    for (int q = cnt[cc]; q < cnt[cc + 1]; q++) {
                        const int j = idx[q];
                        if (j == i) continue;
                        const double px = pi.x - s->pt[j].pos.x, py = pi.y - s->pt[j].pos.y,
                                     pz = pi.z - s->pt[j].pos.z;
                        const double d2 = px * px + py * py + pz * pz;
                        if (d2 > D2 || d2 < 1e-8) continue;
                        const double d = sqrt(d2);
                        const double t = (D - d) / d * 0.5;
                        dx += px * t;
                        dy += py * t;
                        dz += pz * t;
                    }
                }
        d3 q = {pi.x + dx, pi.y + dy, pi.z + dz};
        q.x = q.x < lo[0] ? lo[0] : (q.x > hi[0] ? hi[0] : q.x);
        q.y = q.y < lo[1] ? lo[1] : (q.y > hi[1] ? hi[1] : q.y);
        q.z = q.z < lo[2] ? lo[2] : (q.z > hi[2] ? hi[2] : q.z);
        if (s->p.two_d) q.z = s->p.dims[2] / 2; /* zConst (hashedParticles.cpp:98) */
        np[i] = q;
    }
    for (int i = 0; i < n; i++) s->pt[i].pos = np[i];
    free(np);
    free(fill);
    free(key);
    free(idx);
    free(cnt);
}

static void stage_push_out(sim *s) {
    const double pr = s->p.particle_r;
    d3 lo = {s->cd.x + pr * 1.01, s->cd.y + pr * 1.01, s->cd.z + pr * 1.01};
    d3 hi = {s->dims.x - lo.x, s->dims.y - lo.y, s->dims.z - lo.z};
    const int zc = s->p.two_d;
    const double zval = s->p.dims[2] / 2;
    for (int k = 0; k < s->nobs; k++) {
        const oracle_obstacle *o = &s->obs[k];
        d3 op = obs_pos(o);
        if (is_spherical(o->type)) {
            double r = o->r + pr, r2 = r * r;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < s->n; i++) {
                particle *q = &s->pt[i];
                d3 o2p = {q->pos.x - op.x, q->pos.y - op.y, q->pos.z - op.z};
                double d2 = d3_dot(o2p, o2p);
                if (d2 >= r2) continue;
                double dist = sqrt(d2);
                q->pos.x = op.x + o2p.x / dist * r;
                q->pos.y = op.y + o2p.y / dist * r;
                q->pos.z = op.z + o2p.z / dist * r;
                q->pos.x = clampd(q->pos.x, lo.x, hi.x);
                q->pos.y = clampd(q->pos.y, lo.y, hi.y);
                q->pos.z = zc ? zval : clampd(q->pos.z, lo.z, hi.z);
            }
        }
        if (o->type == ORACLE_OBS_BOX) {
            d3 center = {op.x * s->cdi.x, op.y * s->cdi.y, op.z * s->cdi.z};
            d3 dd = {o->size[0] * s->cdi.x * 0.5, o->size[1] * s->cdi.y * 0.5, o->size[2] * s->cdi.z * 0.5};
            int mn[3], mx[3];
            int gs[3] = {s->nx, s->ny, s->nz};
            for (int a = 0; a < 3; a++) {
                double c = d3_get(&center, a), d = d3_get(&dd, a);
                double l = round(c - d), u = round(c + d);
                mn[a] = (int)(l > 1.0 ? l : 1.0);
                mx[a] = (int)(u < gs[a] - 1.0 ? u : gs[a] - 1.0);
            }
            d3 st = {(double)mn[0] * s->cd.x, (double)mn[1] * s->cd.y, (double)mn[2] * s->cd.z};
            d3 en = {(double)mx[0] * s->cd.x, (double)mx[1] * s->cd.y, (double)mx[2] * s->cd.z};
            st.x -= pr; st.y -= pr; st.z -= pr;
            en.x += pr; en.y += pr; en.z += pr;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < s->n; i++) {
                particle *q = &s->pt[i];
                if ((q->pos.x > en.x || q->pos.x < st.x) || (q->pos.y > en.y || q->pos.y < st.y) ||
                    ((q->pos.z > en.z || q->pos.z < st.z) && !zc))
                    continue;
                int axis = 0;
                double amount = 1e6;
                int axisNum = zc ? 2 : 3;
                for (int p = 0; p < axisNum; p++) {
                    double pp = d3_get(&q->pos, p);
                    if (pp > d3_get(&op, p)) {
                        double tmp = d3_get(&en, p) - pp;
                        if (tmp < fabs(amount)) { amount = tmp; axis = p; }
                    } else {
                        double tmp = d3_get(&st, p) - pp;
                        if (-tmp < fabs(amount)) { amount = tmp; axis = p; }
                    }
                }
                d3_set(&q->pos, axis, d3_get(&q->pos, axis) + amount);
                d3_set(&q->pos, axis, clampd(d3_get(&q->pos, axis), d3_get(&lo, axis), d3_get(&hi, axis)));
            }
        }
    }
}

/* ------------------------------------------------------ grid reset (a8) */

static void reset_grid(sim *s) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->ncell; i++) {
        for (int a = 0; a < 3; a++) { s->v[a][i] = 0.0; s->v2[a][i] = 0.0; s->w[a][i] = 0.0; }
        s->avg[i] = 0.0;
        s->type[i] = ORACLE_AIR;
    }
}

/* ------------------------------------------------------------- P2G (a9) */

/* Simulator::p2gTransfer (simulator.cpp:314-352). */
static void stage_p2g(sim *s) {
    reset_grid(s);
    const int apic = s->p.transfer == ORACLE_APIC;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        const particle *q = &s->pt[i];
        for (int a = 0; a < 3; a++) {
            int b[3];
            face_base(s, q->pos, a, b);
            double va = d3_get(&q->v, a);
            for (int k = 0; k < 8; k++) {
                int x = b[0] + OFF[k][0], y = b[1] + OFF[k][1], z = b[2] + OFF[k][2];
                int ci = cidx(s, x, y, z);
                d3 fp = face_pos(s, a, x, y, z);
                double w = tri_w(fp, q->pos, s->cdi);
                double add;
                if (apic) {
                    d3 p2f = {fp.x - q->pos.x, fp.y - q->pos.y, fp.z - q->pos.z};
                    add = (va + d3_dot(q->c[a], p2f)) * w;
                } else {
                    add = va * w;
                }
#pragma omp atomic
                s->v[a][ci] += add;
#pragma omp atomic
                s->w[a][ci] += w;
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->ncell; i++) {
        for (int a = 0; a < 3; a++) {
            double w = s->w[a][i];
            s->v[a][i] = (w > 1e-6) ? s->v[a][i] / w : 0.0;
        }
    }
}

/* ------------------------------------------------------------ mark (a10) */

/* Simulator::markFluidCellsAndCalculateParticleDensities (simulator.cpp:354-368). */
static void stage_mark(sim *s) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        const particle *q = &s->pt[i];
        int cx = (int)(q->pos.x * s->cdi.x), cy = (int)(q->pos.y * s->cdi.y), cz = (int)(q->pos.z * s->cdi.z);
        s->type[cidx(s, cx, cy, cz)] = ORACLE_WATER;
        int b[3] = {(int)(q->pos.x * s->cdi.x - 0.5), (int)(q->pos.y * s->cdi.y - 0.5),
                    (int)(q->pos.z * s->cdi.z - 0.5)};
        for (int k = 0; k < 8; k++) {
            int x = b[0] + OFF[k][0], y = b[1] + OFF[k][1], z = b[2] + OFF[k][2];
            double w = tri_w(cell_pos(s, x, y, z), q->pos, s->cdi);
#pragma omp atomic
            s->avg[cidx(s, x, y, z)] += w;
        }
    }
}

/* ------------------------------------------------------- obstacles (a11) */

static inline void obstacle_cell(sim *s, int x, int y, int z, d3 speed) {
    int c = cidx(s, x, y, z);
    s->type[c] = ORACLE_SOLID;
    if (s->type[c + s->yz] == ORACLE_WATER) s->v[0][c] = speed.x;
    if (s->type[c - s->yz] == ORACLE_WATER) s->v[0][c - s->yz] = speed.x;
    if (s->type[c + s->nz] == ORACLE_WATER) s->v[1][c] = speed.y;
    if (s->type[c - s->nz] == ORACLE_WATER) s->v[1][c - s->nz] = speed.y;
    if (s->type[c + 1] == ORACLE_WATER) s->v[2][c] = speed.z;
    if (s->type[c - 1] == ORACLE_WATER) s->v[2][c - 1] = speed.z;
}

/* MacGrid::addObstacle (macGrid.cpp:231-292), obstacles in order (simulator.cpp:370-373). */
static void stage_obstacles(sim *s) {
    for (int k = 0; k < s->nobs; k++) {
        const oracle_obstacle *o = &s->obs[k];
        d3 center = {o->pos[0] * s->cdi.x, o->pos[1] * s->cdi.y, o->pos[2] * s->cdi.z};
        d3 speed = obs_speed(o);
        if (o->type == ORACLE_OBS_SPHERE || o->type == ORACLE_OBS_SOURCE) {
            double r = s->cdi.x * o->r, r2 = r * r;
            double lx = center.x - r, ly = center.y - r, lz = center.z - r;
            double ux = center.x + r, uy = center.y + r, uz = center.z + r;
            int mn[3] = {(int)(lx > 1.0 ? lx : 1.0), (int)(ly > 1.0 ? ly : 1.0), (int)(lz > 1.0 ? lz : 1.0)};
            int mx[3] = {(int)(ux < s->nx - 2.0 ? ux : s->nx - 2.0), (int)(uy < s->ny - 2.0 ? uy : s->ny - 2.0),
                         (int)(uz < s->nz - 2.0 ? uz : s->nz - 2.0)};
            for (int x = mn[0]; x <= mx[0]; x++)
                for (int y = mn[1]; y <= mx[1]; y++)
                    for (int z = mn[2]; z <= mx[2]; z++) {
                        d3 c2o = {(x + 0.5) - center.x, (y + 0.5) - center.y, (z + 0.5) - center.z};
                        if (d3_dot(c2o, c2o) < r2) obstacle_cell(s, x, y, z, speed);
                    }
        }
        if (o->type == ORACLE_OBS_BOX) {
            d3 d = {o->size[0] * s->cdi.x * 0.5, o->size[1] * s->cdi.y * 0.5, o->size[2] * s->cdi.z * 0.5};
            int gs[3] = {s->nx, s->ny, s->nz};
            int mn[3], mx[3];
            for (int a = 0; a < 3; a++) {
                double l = round(d3_get(&center, a) - d3_get(&d, a));
                double u = round(d3_get(&center, a) + d3_get(&d, a));
                mn[a] = (int)(l > 1.0 ? l : 1.0);
                mx[a] = (int)(u < gs[a] - 1.0 ? u : gs[a] - 1.0);
            }
            for (int x = mn[0]; x < mx[0]; x++)
                for (int y = mn[1]; y < mx[1]; y++)
                    for (int z = mn[2]; z < mx[2]; z++) obstacle_cell(s, x, y, z, speed);
        }
    }
}

/* ----------------------------------------------------------- walls (a12) */

/* MacGrid::restoreBorderingSolidCellsAndSpeeds (macGrid.cpp:75-140). */
static void walls(sim *s) {
    const int X = s->nx, Y = s->ny, Z = s->nz;
    for (int y = 0; y < Y; y++)
        for (int z = 0; z < Z; z++) {
            s->type[cidx(s, 0, y, z)] = s->type[cidx(s, X - 1, y, z)] = ORACLE_SOLID;
            if (s->type[cidx(s, 1, y, z)] == ORACLE_WATER) s->v[0][cidx(s, 0, y, z)] = 0;
            if (s->type[cidx(s, X - 2, y, z)] == ORACLE_WATER) s->v[0][cidx(s, X - 2, y, z)] = 0;
        }
    for (int x = 0; x < X; x++) {
        for (int z = 0; z < Z; z++) {
            s->type[cidx(s, x, 0, z)] = ORACLE_SOLID;
            if (s->type[cidx(s, x, 1, z)] == ORACLE_WATER) s->v[1][cidx(s, x, 0, z)] = 0;
            if (s->p.top_solid) {
                s->type[cidx(s, x, Y - 1, z)] = ORACLE_SOLID;
                if (s->type[cidx(s, x, Y - 2, z)] == ORACLE_WATER) s->v[1][cidx(s, x, Y - 2, z)] = 0;
            }
        }
        for (int y = 0; y < Y; y++) {
            s->type[cidx(s, x, y, 0)] = s->type[cidx(s, x, y, Z - 1)] = ORACLE_SOLID;
            if (s->type[cidx(s, x, y, 1)] == ORACLE_WATER) s->v[2][cidx(s, x, y, 0)] = 0;
            if (s->type[cidx(s, x, y, Z - 2)] == ORACLE_WATER) s->v[2][cidx(s, x, y, Z - 2)] = 0;
        }
    }
}

/* ------------------------------------------------------- post P2G (a13) */

static void build_fluid_list(sim *s) {
    s->nfluid = 0;
    for (int i = 0; i < s->ncell; i++) s->id[i] = -1;
    for (int x = 1; x < s->nx - 1; x++)
        for (int y = 1; y < s->ny - 1; y++)
            for (int z = 1; z < s->nz - 1; z++) {
                int c = cidx(s, x, y, z);
                if (s->type[c] == ORACLE_WATER) {
                    s->fluid[s->nfluid] = c;
                    s->id[c] = s->nfluid++;
                }
            }
}

/* MacGrid::postP2GUpdate (macGrid.cpp:204-219).  The "cell above" is the raw
 * index c + nz, which for y = ny-1 aliases to cell (x+1, 0, z) as in the
 * reference. */
static void stage_post_p2g(sim *s, double g) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < s->ncell; c++) {
        s->v2[0][c] = s->v[0][c];
        s->v2[1][c] = s->v[1][c];
        s->v2[2][c] = s->v[2][c];
        int above = c + s->nz;
        if (s->type[c] != ORACLE_SOLID && above < s->ncell && s->type[above] != ORACLE_SOLID)
            s->v2[1][c] += g;
    }
    build_fluid_list(s);
}

/* --------------------------------------------------- pressure (a14-a19) */

typedef struct {
    double diag, xw, yw, zw;
} arow;

/* BridsonSolverGrid::applyPreconditioner (bridsonSolverGrid.cpp:126-163). */
static void apply_precon(const sim *s, const arow *A, const double *prec, const double *r, double *q,
                         double *res) {
    const int nf = s->nfluid;
    for (int i = 0; i < nf; i++) {
        int c = s->fluid[i];
        double qneg = 0;
        if (s->type[c - s->yz] == ORACLE_WATER) { int j = s->id[c - s->yz]; qneg += A[j].xw * q[j] * prec[j]; }
        if (s->type[c - s->nz] == ORACLE_WATER) { int j = s->id[c - s->nz]; qneg += A[j].yw * q[j] * prec[j]; }
        if (s->type[c - 1] == ORACLE_WATER) { int j = s->id[c - 1]; qneg += A[j].zw * q[j] * prec[j]; }
        q[i] = (r[i] - qneg) * prec[i];
    }
    for (int i = nf - 1; i >= 0; i--) {
        int c = s->fluid[i];
        double tneg = 0;
        if (s->type[c + s->yz] == ORACLE_WATER) tneg += A[i].xw * res[s->id[c + s->yz]];
        if (s->type[c + s->nz] == ORACLE_WATER) tneg += A[i].yw * res[s->id[c + s->nz]];
        if (s->type[c + 1] == ORACLE_WATER) tneg += A[i].zw * res[s->id[c + 1]];
        res[i] = (q[i] - tneg * prec[i]) * prec[i];
    }
}

/* BridsonSolverGrid::applyAMatrix (bridsonSolverGrid.cpp:165-198). */
static void apply_A(const sim *s, const arow *A, const double *x, double *out) {
    const int nf = s->nfluid;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; i++) {
        int c = s->fluid[i];
        double v = A[i].diag * x[i];
        if (s->type[c + s->yz] == ORACLE_WATER) v += A[i].xw * x[s->id[c + s->yz]];
        if (s->type[c + s->nz] == ORACLE_WATER) v += A[i].yw * x[s->id[c + s->nz]];
        if (s->type[c + 1] == ORACLE_WATER) v += A[i].zw * x[s->id[c + 1]];
        if (s->type[c - s->yz] == ORACLE_WATER) { int j = s->id[c - s->yz]; v += A[j].xw * x[j]; }
        if (s->type[c - s->nz] == ORACLE_WATER) { int j = s->id[c - s->nz]; v += A[j].yw * x[j]; }
        if (s->type[c - 1] == ORACLE_WATER) { int j = s->id[c - 1]; v += A[j].zw * x[j]; }
        out[i] = v;
    }
}

static double dotp(const double *a, const double *b, int n) {
    double r = 0.0;
#pragma omp parallel for reduction(+ : r) schedule(static)
    for (int i = 0; i < n; i++) r += a[i] * b[i];
    return r;
}

/* BridsonSolverGrid::solveIncompressibility (bridsonSolverGrid.cpp:244-293)
 * with calculateRHS (:79-89), calculateAMatrix (:40-77), MIC(0)
 * calculatePreconditioner (:91-124, tau 0.97, sigma 0.25) and
 * applyPressureToVelocities (:295-327).  PCG starts from zero pressure and stops
 * on the absolute max-norm of the recursive residual. */
/* BasicMacGrid::solveIncompressibilityParallel (basicMacGrid.cpp:16-88), the
 * release-build path: max_iters times, every odd-parity WATER cell, then every
 * even one, spreads d = 1.98 (-div v2 [+ density term]) / s over its six faces
 * (s = non-SOLID neighbours; faces towards SOLID neighbours stay).  Cells of
 * one parity share no face, so the result does not depend on the loop order. */
static int stage_sor(sim *s) {
    const double omega = 1.98;
    const int yz = s->yz, nz = s->nz;
    for (int n = 0; n < s->p.max_iters; n++) {
        for (int par = 1; par >= 0; par--) {
#pragma omp parallel for schedule(static)
            for (int x = 1; x < s->nx - 1; x++)
                for (int y = 1; y < s->ny - 1; y++)
                    for (int z = 1; z < nz - 1; z++) {
                        if (((x + y + z) & 1) != par) continue;
                        const int c = x * yz + y * nz + z;
                        if (s->type[c] != ORACLE_WATER) continue;
                        const int s1 = s->type[c + 1] != ORACLE_SOLID, s2 = s->type[c - 1] != ORACLE_SOLID;
                        const int s3 = s->type[c + nz] != ORACLE_SOLID, s4 = s->type[c - nz] != ORACLE_SOLID;
                        const int s5 = s->type[c + yz] != ORACLE_SOLID, s6 = s->type[c - yz] != ORACLE_SOLID;
                        const int ssum = s1 + s2 + s3 + s4 + s5 + s6;
                        if (ssum == 0) continue;
                        double d = -s->v2[0][c] - s->v2[1][c] - s->v2[2][c] + s->v2[0][c - yz] + s->v2[1][c - nz] +
                                   s->v2[2][c - 1] +
                                   (s->p.pressure_enabled ? (s->avg[c] - s->p.average_pressure) * s->p.pressure_k : 0.0);
                        d = d * omega / ssum;
                        if (s1) s->v2[2][c] += d;
                        if (s2) s->v2[2][c - 1] -= d;
                        if (s3) s->v2[1][c] += d;
                        if (s4) s->v2[1][c - nz] -= d;
                        if (s5) s->v2[0][c] += d;
                        if (s6) s->v2[0][c - yz] -= d;
                    }
        }
    }
    s->last_its = s->p.max_iters;
    return s->p.max_iters;
}

static int stage_solve(sim *s, double dt) {
    const int nf = s->nfluid;
    const double tau = 0.97, sig = 0.25;
    for (int i = 0; i < s->ncell; i++) s->pressure[i] = 0.0;
    s->last_its = 0;
    if (nf == 0) return 0;
    double *r = (double *)calloc((size_t)nf, sizeof(double));
    double *p = (double *)calloc((size_t)nf, sizeof(double));
    double *z = (double *)calloc((size_t)nf, sizeof(double));
    double *q = (double *)calloc((size_t)nf, sizeof(double));
    double *sv = (double *)calloc((size_t)nf, sizeof(double));
    double *prec = (double *)calloc((size_t)nf, sizeof(double));
    arow *A = (arow *)calloc((size_t)nf, sizeof(arow));
    const double hs = 1.0 / s->cd.x;
    const int pe = s->p.pressure_enabled;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nf; i++) {
        int c = s->fluid[i];
        r[i] = -hs * (s->v2[0][c] + s->v2[1][c] + s->v2[2][c] - s->v2[0][c - s->yz] - s->v2[1][c - s->nz] -
                      s->v2[2][c - 1]) +
               (pe ? (s->avg[c] - s->p.average_pressure) * s->p.pressure_k : 0.0);
    }
    double total = 0;
    for (int i = 0; i < nf; i++) total += r[i] * r[i];
    int it = 0;
    if (total < 1e-7) goto done;
    {
        const double scale = dt / (s->p.fluid_density * s->cd.x * s->cd.x);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nf; i++) {
            int c = s->fluid[i];
            arow *row = &A[i];
            row->diag = 0; row->xw = 0; row->yw = 0; row->zw = 0;
            const int nb[3] = {s->yz, s->nz, 1};
            double *offd[3] = {&row->xw, &row->yw, &row->zw};
            for (int a = 0; a < 3; a++) {
                uint8_t tp = s->type[c + nb[a]], tn = s->type[c - nb[a]];
                if (tp == ORACLE_WATER) { row->diag += scale; *offd[a] = -scale; }
                else if (tp == ORACLE_AIR) row->diag += scale;
                if (tn != ORACLE_SOLID) row->diag += scale;
            }
        }
        for (int i = 0; i < nf; i++) {
            int c = s->fluid[i];
            double eNeg = 0, eNegTau = 0;
            if (s->type[c - s->yz] == ORACLE_WATER) {
                int j = s->id[c - s->yz];
                double t = A[j].xw * prec[j];
                eNeg += t * t;
                eNegTau += t * (A[j].yw + A[j].zw) * prec[j];
            }
            if (s->type[c - s->nz] == ORACLE_WATER) {
                int j = s->id[c - s->nz];
                double t = A[j].yw * prec[j];
                eNeg += t * t;
                eNegTau += t * (A[j].xw + A[j].zw) * prec[j];
            }
            if (s->type[c - 1] == ORACLE_WATER) {
                int j = s->id[c - 1];
                double t = A[j].zw * prec[j];
                eNeg += t * t;
                eNegTau += t * (A[j].xw + A[j].yw) * prec[j];
            }
            double e = A[i].diag - eNeg - eNegTau * tau;
            if (e < sig * A[i].diag) e = (A[i].diag < 1e-6 ? 1.0 : A[i].diag);
            prec[i] = 1.0 / sqrt(e);
        }
        apply_precon(s, A, prec, r, q, z);
        memcpy(sv, z, (size_t)nf * sizeof(double));
        double sigma = dotp(z, r, nf);
        for (; it < s->p.max_iters; it++) {
            apply_A(s, A, sv, z);
            double alpha = sigma / dotp(sv, z, nf);
            if (alpha != alpha) break;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < nf; i++) {
                p[i] += sv[i] * alpha;
                r[i] += z[i] * -alpha;
            }
            double mx = 0.0;
            for (int i = 0; i < nf; i++)
                if (fabs(r[i]) > mx) mx = fabs(r[i]);
            if (mx < s->p.residual_tol) break;
            apply_precon(s, A, prec, r, q, z);
            double sigmaNew = dotp(z, r, nf);
            if (sigma != sigma) break;
            double beta = sigmaNew / sigma;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < nf; i++) sv[i] = sv[i] * beta + z[i];
            sigma = sigmaNew;
        }
        const double ps = dt / (s->p.fluid_density * s->cd.x);
        for (int i = 0; i < nf; i++) {
            int c = s->fluid[i];
            s->pressure[c] = p[i];
            const int nb[3] = {s->yz, s->nz, 1};
            for (int a = 0; a < 3; a++) {
                int cn = c + nb[a];
                if (s->type[cn] != ORACLE_SOLID) {
                    if (s->type[cn] == ORACLE_AIR) s->v2[a][c] += ps * p[i];
                    else s->v2[a][c] += ps * (p[i] - p[s->id[cn]]);
                }
            }
            for (int a = 0; a < 3; a++) {
                int cn = c - nb[a];
                if (s->type[cn] == ORACLE_AIR) s->v2[a][cn] -= ps * p[i];
            }
        }
    }
done:
    free(r); free(p); free(z); free(q); free(sv); free(prec); free(A);
    s->last_its = it;
    return it;
}

/* ----------------------------------------------------- extrapolate (a20) */

/* MacGrid::extrapolateVelocities (macGrid.cpp:294-336). */
static void stage_extrapolate(sim *s) {
    uint8_t *valid = (uint8_t *)malloc((size_t)s->ncell);
    memset(valid, 100, (size_t)s->ncell);
    for (int i = 0; i < s->nfluid; i++) valid[s->fluid[i]] = 0;
    const int X = s->nx, Y = s->ny, Z = s->nz;
    for (int it = 0; it < 2; it++) {
#pragma omp parallel for schedule(static)
        for (int x = 0; x < X; x++)
            for (int y = 0; y < Y; y++)
                for (int z = 0; z < Z; z++) {
                    int c = cidx(s, x, y, z);
                    if (valid[c] <= it) continue;
                    int cnt = 0;
                    double vs[3] = {0.0, 0.0, 0.0};
                    const int pp[3] = {x, y, z}, lim[3] = {X, Y, Z};
                    for (int a = 0; a < 3; a++)
                        for (int o = 0; o < 2; o++) {
                            int q[3] = {pp[0], pp[1], pp[2]};
                            q[a] += o * 2 - 1;
                            if (q[a] < 0 || q[a] >= lim[a]) continue;
                            int cn = cidx(s, q[0], q[1], q[2]);
                            if (valid[cn] > it) continue;
                            vs[0] += s->v2[0][cn];
                            vs[1] += s->v2[1][cn];
                            vs[2] += s->v2[2][cn];
                            cnt++;
                        }
                    if (cnt > 0) {
                        if (x + 1 < X && s->type[c + s->yz] != ORACLE_WATER) s->v2[0][c] = vs[0] / cnt;
                        if (y + 1 < Y && s->type[c + s->nz] != ORACLE_WATER) s->v2[1][c] = vs[1] / cnt;
                        if (z + 1 < Z && s->type[c + 1] != ORACLE_WATER) s->v2[2][c] = vs[2] / cnt;
                        valid[c] = (uint8_t)(it + 1);
                    }
                }
    }
    free(valid);
}

/* ------------------------------------------------------------- G2P (a21) */

/* Simulator::g2pTransfer (simulator.cpp:375-418). */
static void stage_g2p(sim *s) {
    const int tt = s->p.transfer, twoD = s->p.two_d;
    const float fr = s->p.flip_ratio;
    const double picw = (double)(1 - fr); /* float arithmetic, as in the reference */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        particle *q = &s->pt[i];
        for (int a = 0; a < 3; a++) {
            if (twoD && a == 2) { q->v.z = 0; break; }
            int b[3];
            face_base(s, q->pos, a, b);
            double pic = 0, flip = 0;
            d3 cv = {0, 0, 0};
            for (int k = 0; k < 8; k++) {
                int x = b[0] + OFF[k][0], y = b[1] + OFF[k][1], z = b[2] + OFF[k][2];
                int ci = cidx(s, x, y, z);
                d3 fp = face_pos(s, a, x, y, z);
                double w = tri_w(fp, q->pos, s->cdi);
                double v2 = s->v2[a][ci];
                pic += v2 * w;
                if (tt == ORACLE_FLIP) flip += (v2 - s->v[a][ci]) * w;
                if (tt == ORACLE_APIC) {
                    d3 g = tri_grad(fp, q->pos, s->cdi);
                    cv.x += g.x * v2; cv.y += g.y * v2; cv.z += g.z * v2;
                }
            }
            if (tt == ORACLE_PIC) d3_set(&q->v, a, pic);
            else if (tt == ORACLE_FLIP)
                d3_set(&q->v, a, pic * picw + (flip + d3_get(&q->v, a)) * (double)fr);
            else { d3_set(&q->v, a, pic); q->c[a] = cv; }
        }
    }
}

/* ----------------------------------------------------- stage stepping */

int oracle_stage(void *h, int stage, double dt) {
    sim *s = (sim *)h;
    switch (stage) {
        case ORACLE_STAGE_SPAWN: stage_spawn(s, dt); return 0;
        case ORACLE_STAGE_ADVECT: stage_advect(s, dt); return 0;
        case ORACLE_STAGE_PUSH_APART: stage_push_apart(s); return 0;
        case ORACLE_STAGE_PUSH_OUT: stage_push_out(s); return 0;
        case ORACLE_STAGE_STOP:
            for (int i = 0; i < s->n; i++) { s->pt[i].v.x = 0; s->pt[i].v.y = 0; s->pt[i].v.z = 0; }
            return 0;
        case ORACLE_STAGE_P2G: stage_p2g(s); return 0;
        case ORACLE_STAGE_MARK: stage_mark(s); return 0;
        case ORACLE_STAGE_OBSTACLES: stage_obstacles(s); return 0;
        case ORACLE_STAGE_WALLS: walls(s); return 0;
        case ORACLE_STAGE_POST_P2G:
            stage_post_p2g(s, s->p.gravity_enabled ? (double)s->p.gravity * dt : 0.0);
            return 0;
        case ORACLE_STAGE_SOLVE: return s->p.grid_solver == 1 ? stage_sor(s) : stage_solve(s, dt);
        case ORACLE_STAGE_EXTRAPOLATE: stage_extrapolate(s); return 0;
        case ORACLE_STAGE_G2P: stage_g2p(s); return 0;
        default: return -1;
    }
}

/* Simulator::simulate (simulator.cpp:51-100). */
int oracle_step(void *h, double dt) {
    sim *s = (sim *)h;
    if (s->p.spawning_enabled) stage_spawn(s, dt);
    stage_advect(s, dt);
    if (s->p.push_apart_enabled) stage_push_apart(s);
    stage_push_out(s);
    if (s->p.stop_particles) oracle_stage(s, ORACLE_STAGE_STOP, dt);
    stage_p2g(s);
    stage_mark(s);
    stage_obstacles(s);
    walls(s);
    stage_post_p2g(s, s->p.gravity_enabled ? (double)s->p.gravity * dt : 0.0);
    int its = s->p.grid_solver == 1 ? stage_sor(s) : stage_solve(s, dt);
    stage_extrapolate(s);
    stage_g2p(s);
    return its;
}

void oracle_get_grid(void *h, int field, void *out) {
    sim *s = (sim *)h;
    size_t n = (size_t)s->ncell;
    switch (field) {
        case ORACLE_F_FLAGS: memcpy(out, s->type, n); break;
        case ORACLE_F_AVGPNUM: memcpy(out, s->avg, n * 8); break;
        case ORACLE_F_VX: case ORACLE_F_VY: case ORACLE_F_VZ:
            memcpy(out, s->v[field - ORACLE_F_VX], n * 8); break;
        case ORACLE_F_V2X: case ORACLE_F_V2Y: case ORACLE_F_V2Z:
            memcpy(out, s->v2[field - ORACLE_F_V2X], n * 8); break;
        case ORACLE_F_PRESSURE: memcpy(out, s->pressure, n * 8); break;
        case ORACLE_F_WX: case ORACLE_F_WY: case ORACLE_F_WZ:
            memcpy(out, s->w[field - ORACLE_F_WX], n * 8); break;
        case ORACLE_F_FLUID_ID: memcpy(out, s->id, n * 4); break;
        default: break;
    }
}

void oracle_set_grid(void *h, int field, const void *in) {
    sim *s = (sim *)h;
    size_t n = (size_t)s->ncell;
    switch (field) {
        case ORACLE_F_FLAGS: memcpy(s->type, in, n); build_fluid_list(s); break;
        case ORACLE_F_AVGPNUM: memcpy(s->avg, in, n * 8); break;
        case ORACLE_F_VX: case ORACLE_F_VY: case ORACLE_F_VZ:
            memcpy(s->v[field - ORACLE_F_VX], in, n * 8); break;
        case ORACLE_F_V2X: case ORACLE_F_V2Y: case ORACLE_F_V2Z:
            memcpy(s->v2[field - ORACLE_F_V2X], in, n * 8); break;
        case ORACLE_F_WX: case ORACLE_F_WY: case ORACLE_F_WZ:
            memcpy(s->w[field - ORACLE_F_WX], in, n * 8); break;
        default: break;
    }
}

int oracle_fluid_count(void *h) { return ((sim *)h)->nfluid; }

int oracle_last_iterations(void *h) { return ((sim *)h)->last_its; }
