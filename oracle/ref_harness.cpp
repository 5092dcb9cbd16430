// ref_harness.cpp -- drives the reference's own, unmodified Simulator sources
// (dkiovics/fluid_simulator src/Simulator/simulator/**) through the oracle C
// interface in oracle_api.h.  Test infrastructure only: built into
// oracle/_ref/libfsim_ref.so by oracle/Makefile, never linked by the product.
//
// Observation hooks, all without editing the reference:
//  * ProbeGrid derives from BridsonSolverGrid (bridsonSolverGrid.h:12) and
//    overrides the public virtual solveIncompressibility (macGrid.h:165).  It
//    snapshots v2 before the base solve and recovers the solved pressure from
//    the linear velocity update of applyPressureToVelocities
//    (bridsonSolverGrid.cpp:295-327): an AIR-adjacent face moves by +-scale*p_i,
//    a fluid-fluid face by scale*(p_i - p_j); a breadth-first walk from the
//    AIR-adjacent cells recovers every p_i of components that touch air.
//  * Single stages call the Simulator/MacGrid member functions directly; the
//    access specifiers of the reference headers are opened for this
//    translation unit only (class layout is unaffected).
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>
#include <omp.h>

#include <glm/glm.hpp>

#define private public
#define protected public
#include "simulator/simulator.h"
#include "simulator/macGrid/bridsonSolverGrid.h"
#include "simulator/macGrid/basicMacGrid.h"
#include "simulator/particles/hashedParticles.h"
#include "simulator/macGrid/obstacles.hpp"
#undef private
#undef protected

#include "oracle_api.h"

using namespace genericfsim;

namespace {

class ProbeGrid : public macgrid::BridsonSolverGrid {
public:
    ProbeGrid(const glm::dvec3& dims, float res, bool twoD, double rho)
        : macgrid::BridsonSolverGrid(dims, res, twoD, rho), dims0(dims), res0(res) {}

    glm::dvec3 dims0;  // constructor arguments, to build an identical BasicMacGrid
    double res0;

    std::vector<double> pressure;
    int lastIterations = 0;
    int gridSolver = 0;  // 1: run the reference's BasicMacGrid SOR instead

    // BasicMacGrid::solveIncompressibility (basicMacGrid.cpp:5-12) on a copy of
    // this grid's cell types, v2 and densities; v2 comes back
    int solveBasic(bool parallel, double dt) {
        macgrid::BasicMacGrid basic(dims0, res0, twoD);
        basic.pressureEnabled = pressureEnabled;
        basic.pressureK = pressureK;
        basic.averagePressure = averagePressure;
        basic.incompressibilityMaxIterationCount = incompressibilityMaxIterationCount;
        for (int i = 0; i < cellCount; i++) {
            basic.rawCells[i].type = rawCells[i].type;
            basic.rawCells[i].avgPNum = rawCells[i].avgPNum.load();
            for (int a = 0; a < 3; a++) basic.rawCells[i].faces[a].v2 = rawCells[i].faces[a].v2;
        }
        const int its = basic.solveIncompressibility(parallel, dt);
        for (int i = 0; i < cellCount; i++)
            for (int a = 0; a < 3; a++) rawCells[i].faces[a].v2 = basic.rawCells[i].faces[a].v2;
        pressure.assign(cellCount, 0.0);
        return its;
    }

    int solveIncompressibility(bool parallel, double dt) override {
        if (gridSolver == 1) return lastIterations = solveBasic(parallel, dt);
        const int n = cellCount;
        std::vector<double> before[3];
        for (int a = 0; a < 3; a++) {
            before[a].resize(n);
            for (int i = 0; i < n; i++) before[a][i] = rawCells[i].faces[a].v2;
        }
        lastIterations = macgrid::BridsonSolverGrid::solveIncompressibility(parallel, dt);
        recoverPressure(before, dt);
        return lastIterations;
    }

    void recoverPressure(const std::vector<double> (&before)[3], double dt) {
        const int n = cellCount;
        const double scale = dt / (fluidDensity * cellD.x);
        pressure.assign(n, 0.0);
        std::vector<char> known(n, 0);
        auto idx = [&](int x, int y, int z) { return (x * gridSize.y + y) * gridSize.z + z; };
        auto delta = [&](int a, int i) { return rawCells[i].faces[a].v2 - before[a][i]; };
        using CT = macgrid::MacGridCell::CellType;
        std::deque<glm::ivec3> queue;
        for (const auto& p : fluidCellPositions) {
            const int i = idx(p.x, p.y, p.z);
            pressure[i] = std::numeric_limits<double>::quiet_NaN();
        }
        for (const auto& p : fluidCellPositions) {
            const int i = idx(p.x, p.y, p.z);
            for (int a = 0; a < 3 && !known[i]; a++) {
                glm::ivec3 q = p;
                q[a] += 1;
                if (cell(q).type == CT::AIR) {
                    pressure[i] = delta(a, i) / scale;
                    known[i] = 1;
                    break;
                }
                q[a] -= 2;
                if (cell(q).type == CT::AIR) {
                    pressure[i] = -delta(a, idx(q.x, q.y, q.z)) / scale;
                    known[i] = 1;
                }
            }
            if (known[i]) queue.push_back(p);
        }
        while (!queue.empty()) {
            glm::ivec3 p = queue.front();
            queue.pop_front();
            const int i = idx(p.x, p.y, p.z);
            for (int a = 0; a < 3; a++) {
                glm::ivec3 q = p;
                q[a] += 1;
                int j = idx(q.x, q.y, q.z);
                if (cell(q).type == CT::WATER && !known[j]) {
                    pressure[j] = pressure[i] - delta(a, i) / scale;
                    known[j] = 1;
                    queue.push_back(q);
                }
                q[a] -= 2;
                j = idx(q.x, q.y, q.z);
                if (cell(q).type == CT::WATER && !known[j]) {
                    pressure[j] = pressure[i] + delta(a, j) / scale;
                    known[j] = 1;
                    queue.push_back(q);
                }
            }
        }
    }

    void rebuildFluidList() {
        fluidCellPositions.clear();
        for (int x = 1; x < gridSize.x - 1; x++)
            for (int y = 1; y < gridSize.y - 1; y++)
                for (int z = 1; z < gridSize.z - 1; z++) {
                    auto& c = cell(x, y, z);
                    if (c.type == macgrid::MacGridCell::CellType::WATER) {
                        fluidCellPositions.push_back(glm::ivec3(x, y, z));
                        c.id = (int)fluidCellPositions.size() - 1;
                    }
                }
    }
};

struct Handle {
    oracle_params params;
    std::shared_ptr<ProbeGrid> grid;
    std::shared_ptr<particles::HashedParticles> parts;
    std::unique_ptr<simulator::Simulator> sim;
};

simulator::Simulator::SimulatorConfig makeConfig(const oracle_params* p) {
    simulator::Simulator::SimulatorConfig c;
    c.transferType = p->transfer == ORACLE_PIC    ? simulator::Simulator::P2G2PType::PIC
                     : p->transfer == ORACLE_FLIP ? simulator::Simulator::P2G2PType::FLIP
                                                  : simulator::Simulator::P2G2PType::APIC;
    c.flipRatio = p->flip_ratio;
    c.gravity = p->gravity;
    c.gravityEnabled = p->gravity_enabled != 0;
    c.pushApartEnabled = p->push_apart_enabled != 0;
    c.pushParticlesApartEnabled = p->push_apart_enabled != 0;
    c.particleSpawningEnabled = p->spawning_enabled != 0;
    c.particleDespawningEnabled = p->despawning_enabled != 0;
    c.stopParticles = p->stop_particles != 0;
    return c;
}

void applyGridParams(Handle* h) {
    const oracle_params* p = &h->params;
    h->grid->isTopOfContainerSolid = p->top_solid != 0;
    h->grid->pressureK = p->pressure_k;
    h->grid->averagePressure = p->average_pressure;
    h->grid->incompressibilityMaxIterationCount = p->max_iters;
    h->grid->pressureEnabled = p->pressure_enabled != 0;
    h->grid->fluidDensity = p->fluid_density;
    h->grid->residualTolerance = p->residual_tol;
    h->grid->gridSolver = p->grid_solver;
}

void writeParticles(Handle* h, int n, const double* pos, const double* vel, const double* c) {
    if (h->parts->getParticleNum() != n) h->parts->setParticleNum(n);
    for (int i = 0; i < n; i++) {
        particles::Particle& q = h->parts->getParticleAt(i);
        q.pos = glm::dvec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        q.v = glm::dvec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        for (int a = 0; a < 3; a++)
            q.c[a] = c ? glm::dvec3(c[9 * i + 3 * a], c[9 * i + 3 * a + 1], c[9 * i + 3 * a + 2])
                       : glm::dvec3(0.0);
    }
}

}  // namespace

extern "C" {

void* oracle_create(const oracle_params* p, int n, const double* pos, const double* vel,
                    const double* c) {
    auto* h = new Handle();
    h->params = *p;
    const glm::dvec3 dims(p->dims[0], p->dims[1], p->dims[2]);
    h->grid = std::make_shared<ProbeGrid>(dims, (float)p->resolution, p->two_d != 0,
                                          p->fluid_density);
    applyGridParams(h);
    h->parts = std::make_shared<particles::HashedParticles>(
        n, p->particle_r, h->grid->dimensions, h->grid->cellD, p->two_d != 0, dims.z / 2);
    writeParticles(h, n, pos, vel, c);
    h->sim = std::make_unique<simulator::Simulator>(makeConfig(p), h->parts, h->grid);
    return h;
}

void oracle_destroy(void* hv) { delete static_cast<Handle*>(hv); }

void oracle_set_threads(int n) { omp_set_num_threads(n); }

void oracle_grid_size(void* hv, int* n3) {
    auto* h = static_cast<Handle*>(hv);
    n3[0] = h->grid->gridSize.x;
    n3[1] = h->grid->gridSize.y;
    n3[2] = h->grid->gridSize.z;
}

void oracle_cell_size(void* hv, double* h3) {
    auto* h = static_cast<Handle*>(hv);
    h3[0] = h->grid->cellD.x;
    h3[1] = h->grid->cellD.y;
    h3[2] = h->grid->cellD.z;
}

int oracle_num_particles(void* hv) { return static_cast<Handle*>(hv)->parts->getParticleNum(); }

void oracle_get_particles(void* hv, double* pos, double* vel, double* c) {
    auto* h = static_cast<Handle*>(hv);
    const int n = h->parts->getParticleNum();
    for (int i = 0; i < n; i++) {
        const particles::Particle& q = h->parts->getParticleAt(i);
        for (int a = 0; a < 3; a++) {
            if (pos) pos[3 * i + a] = q.pos[a];
            if (vel) vel[3 * i + a] = q.v[a];
            if (c)
                for (int b = 0; b < 3; b++) c[9 * i + 3 * a + b] = q.c[a][b];
        }
    }
}

void oracle_set_particles(void* hv, int n, const double* pos, const double* vel, const double* c) {
    writeParticles(static_cast<Handle*>(hv), n, pos, vel, c);
}

void oracle_set_params(void* hv, const oracle_params* p) {
    auto* h = static_cast<Handle*>(hv);
    h->params = *p;
    applyGridParams(h);
    h->sim->config = makeConfig(p);
}

void oracle_set_obstacles(void* hv, int n, const oracle_obstacle* obs) {
    auto* h = static_cast<Handle*>(hv);
    h->sim->obstacles.clear();
    for (int i = 0; i < n; i++) {
        const oracle_obstacle& o = obs[i];
        if (o.type > ORACLE_OBS_SINK) continue;  // extensions have no reference counterpart
        const glm::dvec3 pos(o.pos[0], o.pos[1], o.pos[2]);
        obstacle::Obstacle* made = nullptr;
        switch (o.type) {
            case ORACLE_OBS_SPHERE: made = new obstacle::SphericalObstacle(o.r, pos); break;
            case ORACLE_OBS_BOX:
                made = new obstacle::RectengularObstacle(glm::dvec3(o.size[0], o.size[1], o.size[2]), pos);
                break;
            case ORACLE_OBS_SOURCE: {
                auto* s = new obstacle::SphericalParticleSource(o.r, o.spawn_rate, o.spawn_speed, pos);
                s->lastSpawnFraction = o.last_spawn_fraction;
                made = s;
                break;
            }
            default: made = new obstacle::SphericalParticleSink(o.r, pos); break;
        }
        made->prevPos = glm::dvec3(o.prev_pos[0], o.prev_pos[1], o.prev_pos[2]);
        made->speed = glm::dvec3(o.speed[0], o.speed[1], o.speed[2]);
        h->sim->obstacles.push_back(std::unique_ptr<obstacle::Obstacle>(made));
    }
}

int oracle_get_obstacles(void* hv, int cap, oracle_obstacle* obs) {
    auto* h = static_cast<Handle*>(hv);
    int n = (int)h->sim->obstacles.size();
    for (int i = 0; i < n && i < cap; i++) {
        obstacle::Obstacle* o = h->sim->obstacles[i].get();
        oracle_obstacle& out = obs[i];
        std::memset(&out, 0, sizeof(out));
        for (int a = 0; a < 3; a++) {
            out.pos[a] = o->pos[a];
            out.prev_pos[a] = o->prevPos[a];
            out.speed[a] = o->speed[a];
        }
        if (auto* s = dynamic_cast<obstacle::SphericalParticleSource*>(o)) {
            out.type = ORACLE_OBS_SOURCE;
            out.r = s->r;
            out.spawn_rate = s->particleSpawnRate;
            out.spawn_speed = s->particleSpawnSpeed;
            out.last_spawn_fraction = s->lastSpawnFraction;
        } else if (auto* k = dynamic_cast<obstacle::SphericalParticleSink*>(o)) {
            out.type = ORACLE_OBS_SINK;
            out.r = k->r;
        } else if (auto* sp = dynamic_cast<obstacle::SphericalObstacle*>(o)) {
            out.type = ORACLE_OBS_SPHERE;
            out.r = sp->r;
        } else if (auto* b = dynamic_cast<obstacle::RectengularObstacle*>(o)) {
            out.type = ORACLE_OBS_BOX;
            for (int a = 0; a < 3; a++) out.size[a] = b->size[a];
        }
    }
    return n;
}

int oracle_step(void* hv, double dt) {
    auto* h = static_cast<Handle*>(hv);
    h->grid->lastIterations = 0;
    h->sim->simulate(dt);
    return h->grid->lastIterations;
}

int oracle_stage(void* hv, int stage, double dt) {
    auto* h = static_cast<Handle*>(hv);
    simulator::Simulator& s = *h->sim;
    const bool par = true;  // the release-build setting; OMP thread count decides
    switch (stage) {
        case ORACLE_STAGE_SPAWN: s.spawnParticles(dt); break;
        case ORACLE_STAGE_ADVECT: s.advectParticles(par, dt); break;
        case ORACLE_STAGE_PUSH_APART:
            h->parts->updateParticleIntersectionHash(par);
            h->parts->pushParticlesApart(par);
            break;
        case ORACLE_STAGE_PUSH_OUT: s.pushParticlesOutOfObstacles(par); break;
        case ORACLE_STAGE_STOP:
            h->parts->forEach(par, [](particles::Particle& q, int) { q.v = glm::dvec3(0.0); });
            break;
        case ORACLE_STAGE_P2G:
            h->grid->resetGridValues(par);
            s.p2gTransfer(par, dt);
            break;
        case ORACLE_STAGE_MARK: s.markFluidCellsAndCalculateParticleDensities(par); break;
        case ORACLE_STAGE_OBSTACLES: s.addObstaclesToGrid(par); break;
        case ORACLE_STAGE_WALLS: h->grid->restoreBorderingSolidCellsAndSpeeds(par); break;
        case ORACLE_STAGE_POST_P2G:
            h->grid->postP2GUpdate(par, s.config.gravityEnabled ? s.config.gravity * dt : 0.0);
            break;
        case ORACLE_STAGE_SOLVE: return h->grid->solveIncompressibility(par, dt);
        case ORACLE_STAGE_EXTRAPOLATE: h->grid->extrapolateVelocities(par); break;
        case ORACLE_STAGE_G2P: s.g2pTransfer(par); break;
        default: return -1;
    }
    return 0;
}

void oracle_get_grid(void* hv, int field, void* out) {
    auto* h = static_cast<Handle*>(hv);
    ProbeGrid& g = *h->grid;
    const int n = g.cellCount;
    for (int i = 0; i < n; i++) {
        const auto& c = g.rawCells[i];
        switch (field) {
            case ORACLE_F_FLAGS: static_cast<uint8_t*>(out)[i] = (uint8_t)c.type; break;
            case ORACLE_F_AVGPNUM: static_cast<double*>(out)[i] = c.avgPNum.load(); break;
            case ORACLE_F_VX: case ORACLE_F_VY: case ORACLE_F_VZ:
                static_cast<double*>(out)[i] = c.faces[field - ORACLE_F_VX].v.load();
                break;
            case ORACLE_F_V2X: case ORACLE_F_V2Y: case ORACLE_F_V2Z:
                static_cast<double*>(out)[i] = c.faces[field - ORACLE_F_V2X].v2;
                break;
            case ORACLE_F_PRESSURE:
                static_cast<double*>(out)[i] = g.pressure.empty() ? 0.0 : g.pressure[i];
                break;
            case ORACLE_F_WX: case ORACLE_F_WY: case ORACLE_F_WZ:
                static_cast<double*>(out)[i] = c.faces[field - ORACLE_F_WX].particleWeightSum.load();
                break;
            case ORACLE_F_FLUID_ID:
                static_cast<int32_t*>(out)[i] = -1;
                break;
        }
    }
    if (field == ORACLE_F_FLUID_ID) {
        for (const auto& p : g.fluidCellPositions)
            static_cast<int32_t*>(out)[(p.x * g.gridSize.y + p.y) * g.gridSize.z + p.z] = g.cell(p).id;
    }
}

void oracle_set_grid(void* hv, int field, const void* in) {
    auto* h = static_cast<Handle*>(hv);
    ProbeGrid& g = *h->grid;
    const int n = g.cellCount;
    using CT = macgrid::MacGridCell::CellType;
    for (int i = 0; i < n; i++) {
        auto& c = g.rawCells[i];
        switch (field) {
            case ORACLE_F_FLAGS: c.type = (CT) static_cast<const uint8_t*>(in)[i]; break;
            case ORACLE_F_AVGPNUM: c.avgPNum = static_cast<const double*>(in)[i]; break;
            case ORACLE_F_VX: case ORACLE_F_VY: case ORACLE_F_VZ:
                c.faces[field - ORACLE_F_VX].v = static_cast<const double*>(in)[i];
                break;
            case ORACLE_F_V2X: case ORACLE_F_V2Y: case ORACLE_F_V2Z:
                c.faces[field - ORACLE_F_V2X].v2 = static_cast<const double*>(in)[i];
                break;
            case ORACLE_F_WX: case ORACLE_F_WY: case ORACLE_F_WZ:
                c.faces[field - ORACLE_F_WX].particleWeightSum = static_cast<const double*>(in)[i];
                break;
            default: break;
        }
    }
    if (field == ORACLE_F_FLAGS) g.rebuildFluidList();
}

int oracle_fluid_count(void* hv) { return (int)static_cast<Handle*>(hv)->grid->fluidCellPositions.size(); }

int oracle_last_iterations(void* hv) { return static_cast<Handle*>(hv)->grid->lastIterations; }

}  // extern "C"
