// fsim_facade.hpp -- the reference's Simulator-level C++ interface over the
// GB300 step library (include/fsim.h).
//
// The reference's SimulationManager (src/Simulator/manager/simulationManager.cpp)
// owns a Simulator, a MacGrid (BridsonSolverGrid) and a HashedParticles and
// drives them through the classes and members declared in
//   src/Simulator/simulator/simulator.h:15-84          (Simulator, SimulatorConfig, P2G2PType)
//   src/Simulator/simulator/macGrid/macGrid.h:17-182    (MacGrid public members)
//   src/Simulator/simulator/macGrid/macGridCell.h:8-54  (MacGridCell)
//   src/Simulator/simulator/macGrid/bridsonSolverGrid.h:11-17
//   src/Simulator/simulator/particles/hashedParticles.h:30-177, particle.h:8-12
//   src/Simulator/simulator/macGrid/obstacles.hpp:7-65  (Obstacle family)
// This header declares the same namespaces, class names, constructors, public
// fields and methods, so the manager compiles against it in place of those
// headers.  Simulator::simulate runs one fsim_step on the GPU.
//
// State lives on the device.  The host objects keep mirrors that are
// downloaded lazily: the first host access to a particle or a cell after a
// step copies the state back, and any non-const access marks the particles as
// edited so the next simulate() uploads them again.  Returned references stay
// valid until the next simulate().
//
// Parts of the reference interface that only the reference's own Simulator
// uses internally (grid reset, P2G helpers, the intersection hash) are not
// declared; the stencil accessors getFacesAround / getCellsAround and the
// trilinear helpers of util/interpolation.h are, since callers of the
// Simulator (the manager's gfx fill) use them.  Push-apart runs with the library's
// deterministic (Jacobi) semantics.  BasicMacGrid selects the library's SOR
// solver.  Default particle positions of HashedParticles
// use a SplitMix64 generator instead of std::rand.
//
// Requires glm (glm::dvec3, glm::ivec3) and C++17.
#pragma once

#include <glm/glm.hpp>

#include <cmath>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include <array>
#include <atomic>

#include "fsim.h"

namespace genericfsim {

// ---------------------------------------------------------------- obstacles
namespace obstacle {

struct Obstacle {
    glm::dvec3 pos;
    glm::dvec3 prevPos;
    glm::dvec3 speed = glm::dvec3(0, 0, 0);

    Obstacle(const glm::dvec3& pos = glm::dvec3(0, 0, 0)) : pos(pos), prevPos(pos) {}
    virtual ~Obstacle() = default;

    void setNewPos(const glm::dvec3& p) {
        prevPos = pos;
        pos = p;
    }
    void calculateSpeed(double dt) { speed = (pos - prevPos) / dt; }
    virtual Obstacle* clone() = 0;
};

struct RectengularObstacle : public Obstacle {
    const glm::dvec3 size;
    RectengularObstacle(const glm::dvec3& size, const glm::dvec3& pos = glm::dvec3(0, 0, 0))
        : Obstacle(pos), size(size) {}
    Obstacle* clone() override { return new RectengularObstacle(*this); }
};

struct SphericalObstacle : public Obstacle {
    const double r;
    SphericalObstacle(double r, const glm::dvec3& pos = glm::dvec3(0, 0, 0)) : Obstacle(pos), r(r) {}
    Obstacle* clone() override { return new SphericalObstacle(*this); }
};

struct SphericalParticleSource : public SphericalObstacle {
    const double particleSpawnRate;
    const double particleSpawnSpeed;
    double lastSpawnFraction = 0;
    SphericalParticleSource(double r, double particleSpawnRate, double particleSpawnSpeed,
                            const glm::dvec3& pos = glm::dvec3(0, 0, 0))
        : SphericalObstacle(r, pos), particleSpawnRate(particleSpawnRate), particleSpawnSpeed(particleSpawnSpeed) {}
    Obstacle* clone() override { return new SphericalParticleSource(*this); }
};

struct SphericalParticleSink : public SphericalObstacle {
    SphericalParticleSink(double r, const glm::dvec3& pos = glm::dvec3(0, 0, 0)) : SphericalObstacle(r, pos) {}
    Obstacle* clone() override { return new SphericalParticleSink(*this); }
};

// Extensions of the GPU library (no reference counterpart): a horizontal disc
// emitting 8 jittered particles per covered cell and step with velocity
// (0, particleSpawnSpeed, 0), and an axis-aligned box that deletes particles.
struct DiscParticleSource : public Obstacle {
    const double r;
    const double particleSpawnSpeed;
    DiscParticleSource(double r, double particleSpawnSpeed, const glm::dvec3& pos = glm::dvec3(0, 0, 0))
        : Obstacle(pos), r(r), particleSpawnSpeed(particleSpawnSpeed) {}
    Obstacle* clone() override { return new DiscParticleSource(*this); }
};

struct RectengularParticleSink : public Obstacle {
    const glm::dvec3 size;
    RectengularParticleSink(const glm::dvec3& size, const glm::dvec3& pos = glm::dvec3(0, 0, 0))
        : Obstacle(pos), size(size) {}
    Obstacle* clone() override { return new RectengularParticleSink(*this); }
};

}  // namespace obstacle

// ---------------------------------------------------------------- particles
namespace particles {

struct Particle {
    glm::dvec3 pos;
    glm::dvec3 v;
    glm::dvec3 c[3];
};

}  // namespace particles

namespace facade_detail {

inline void check(int rc, fsim_ctx* ctx, const char* what) {
    if (rc != FSIM_OK) {
        std::string msg = std::string(what) + " failed (" + std::to_string(rc) + ")";
        if (ctx) msg += std::string(": ") + fsim_last_error(ctx);
        throw std::runtime_error(msg);
    }
}

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline double uniform(uint64_t& state, double lo, double hi) {
    state = splitmix64(state);
    return lo + (hi - lo) * (double)(state >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace facade_detail

namespace simulator {
class Simulator;
}

namespace particles {

class HashedParticles {
public:
    // Reference: num particles at random positions in the upper half of the box
    // (hashedParticles.cpp:23-42).
    HashedParticles(int num, double r, glm::dvec3 dimensions, glm::dvec3 cellD, bool zConst, double z)
        : z(z), zConst(zConst), dimensions(dimensions), cellD(cellD), r(r) {
        particles.reserve(num);
        for (int p = 0; p < num; p++) {
            Particle q;
            q.pos = glm::dvec3(
                facade_detail::uniform(rng, dimensions.x * 0.5 + cellD.x, dimensions.x - 1.1 * r - cellD.x),
                facade_detail::uniform(rng, dimensions.y * 0.5 + cellD.y, dimensions.y - 1.1 * r - cellD.y),
                zConst ? z : facade_detail::uniform(rng, dimensions.z * 0.5 + cellD.z, dimensions.z - 1.1 * r - cellD.z));
            q.v = glm::dvec3(0, 0, 0);
            q.c[0] = q.c[1] = q.c[2] = glm::dvec3(0, 0, 0);
            particles.push_back(q);
        }
    }

    void forEach(bool /*parallel*/, std::function<void(Particle&, int)>&& lambda) {
        pull();
        edited = true;
        for (int i = 0; i < (int)particles.size(); i++) lambda(particles[i], i);
    }

    // Reference: truncates, or appends particles at random positions (hashedParticles.cpp:132-151).
    void setParticleNum(int num) {
        pull();
        edited = true;
        if (num < (int)particles.size()) particles.resize(num);
        while ((int)particles.size() < num) {
            Particle q;
            q.pos = glm::dvec3(facade_detail::uniform(rng, 1.1 * r + cellD.x, dimensions.x - 1.1 * r - cellD.x),
                               facade_detail::uniform(rng, 1.1 * r + cellD.y, dimensions.y - 1.1 * r - cellD.y),
                               zConst ? z : facade_detail::uniform(rng, 1.1 * r + cellD.z, dimensions.z - 1.1 * r - cellD.z));
            q.v = glm::dvec3(0, 0, 0);
            q.c[0] = q.c[1] = q.c[2] = glm::dvec3(0, 0, 0);
            particles.push_back(q);
        }
    }

    Particle& getParticleAt(int idx) {
        pull();
        edited = true;
        return particles.at(idx);
    }

    int getParticleNum() const {
        if (device && !host_valid) {
            int64_t n = 0;
            facade_detail::check(fsim_num_particles(device, &n), device, "fsim_num_particles");
            return (int)n;
        }
        return (int)particles.size();
    }

    double getParticleR() const { return r; }
    void setParticleR(double nr) { r = nr; }

    void updateGridParams(const glm::dvec3& newCellD, const glm::dvec3& newDimensions) {
        cellD = newCellD;
        dimensions = newDimensions;
    }

    void addParticles(std::vector<Particle>&& add) {
        pull();
        edited = true;
        particles.insert(particles.end(), add.begin(), add.end());
    }

    // Reference: removes the given indices, keeping the order of the rest (hashedParticles.cpp:158-172).
    void removeParticles(std::vector<int>&& ids) {
        pull();
        edited = true;
        std::vector<char> gone(particles.size(), 0);
        for (int i : ids)
            if (i >= 0 && i < (int)particles.size()) gone[i] = 1;
        size_t w = 0;
        for (size_t p = 0; p < particles.size(); p++)
            if (!gone[p]) particles[w++] = particles[p];
        particles.resize(w);
    }

    // Reference: hashedParticles.cpp:64-107; the library's deterministic (Jacobi)
    // push-apart pass on the bound context (FSIM_STAGE_PUSH_APART)
    void pushParticlesApart(bool /*parallel*/) {
        if (!device) throw std::runtime_error("pushParticlesApart: the particles are not bound to a Simulator");
        if (edited) push(device);
        facade_detail::check(fsim_stage(device, FSIM_STAGE_PUSH_APART, 0.0, nullptr), device,
                             "fsim_stage(PUSH_APART)");
        host_valid = false;
    }

    const double z;
    const bool zConst;

private:
    friend class simulator::Simulator;

    // device -> host mirror when the device holds newer state
    void pull() {
        if (!device || host_valid) return;
        int64_t n = 0;
        facade_detail::check(fsim_num_particles(device, &n), device, "fsim_num_particles");
        std::vector<float> pos((size_t)n * 3), vel((size_t)n * 3), c((size_t)n * 9);
        int64_t got = 0;
        facade_detail::check(fsim_get_particles(device, pos.data(), vel.data(), c.data(), n, &got, FSIM_HOST), device,
                             "fsim_get_particles");
        particles.resize((size_t)got);
        for (int64_t i = 0; i < got; i++) {
            Particle& q = particles[(size_t)i];
            q.pos = glm::dvec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
            q.v = glm::dvec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
            for (int a = 0; a < 3; a++) q.c[a] = glm::dvec3(c[9 * i + 3 * a], c[9 * i + 3 * a + 1], c[9 * i + 3 * a + 2]);
        }
        host_valid = true;
    }

    // host -> device (FP32, the library's storage precision)
    void push(fsim_ctx* ctx) {
        const size_t n = particles.size();
        std::vector<float> pos(n * 3), vel(n * 3), c(n * 9);
        for (size_t i = 0; i < n; i++) {
            const Particle& q = particles[i];
            for (int a = 0; a < 3; a++) {
                pos[3 * i + a] = (float)q.pos[a];
                vel[3 * i + a] = (float)q.v[a];
                for (int b = 0; b < 3; b++) c[9 * i + 3 * a + b] = (float)q.c[a][b];
            }
        }
        facade_detail::check(fsim_set_particles(ctx, pos.data(), vel.data(), c.data(), (int64_t)n, FSIM_HOST), ctx,
                             "fsim_set_particles");
        device = ctx;
        host_valid = true;
        edited = false;
    }

    std::vector<Particle> particles;
    glm::dvec3 dimensions;
    glm::dvec3 cellD;
    double r;
    uint64_t rng = 0x5eed;
    fsim_ctx* device = nullptr;  // context holding the newest state (set by Simulator)
    bool host_valid = true;
    bool edited = true;
};

}  // namespace particles

// ---------------------------------------------------------------- grid
namespace macgrid {

struct MacGridCell {
    struct Face {
        std::atomic<double> v = 0.0;
        double v2 = 0;
        std::atomic<double> particleWeightSum = 0.0;
        const glm::dvec3 pos;

        Face(glm::dvec3 pos) : pos(std::move(pos)) {}
        Face(const Face& face) : v(face.v.load()), v2(face.v2), particleWeightSum(face.particleWeightSum.load()), pos(face.pos) {}
        const Face& operator=(const Face& face) {
            v = face.v.load();
            v2 = face.v2;
            particleWeightSum = face.particleWeightSum.load();
            return *this;
        }
    };

    struct FaceRef {
        Face& face;
    };

    enum class CellType { WATER, AIR, SOLID };

    Face faces[3];
    const glm::dvec3 pos;
    CellType type = CellType::AIR;
    std::atomic<double> avgPNum = 0.0;
    int id = 0;

    MacGridCell(const Face& fx, const Face& fy, const Face& fz, const glm::dvec3& pos) : faces{fx, fy, fz}, pos(pos) {}
    MacGridCell(const MacGridCell& cell)
        : faces{cell.faces[0], cell.faces[1], cell.faces[2]}, pos(cell.pos), type(cell.type),
          avgPNum(cell.avgPNum.load()), id(cell.id) {}
};

struct MacGridCellRef {
    MacGridCell& cell;
};

class MacGrid {
public:
    // Reference geometry (macGrid.cpp:9-33): cellD = 1/resolution, gridSize =
    // trunc(dims / cellD), border cells are the walls.
    MacGrid(glm::dvec3 targetDimensions, double resolution, bool twoD)
        : cellD(1 / resolution, 1 / resolution, twoD ? targetDimensions.z / 3 : 1 / resolution),
          cellDInv(1.0 / cellD),
          gridSize(targetDimensions.x / cellD.x, targetDimensions.y / cellD.y, twoD ? 3 : targetDimensions.z / cellD.z),
          dimensions(gridSize.x * cellD.x, gridSize.y * cellD.y, twoD ? targetDimensions.z : gridSize.z * cellD.z),
          twoD(twoD), resolution(resolution), requestedDimensions(targetDimensions) {
        rawCells.reserve((size_t)gridSize.x * gridSize.y * gridSize.z);
        for (int x = 0; x < gridSize.x; x++)
            for (int y = 0; y < gridSize.y; y++)
                for (int z = 0; z < gridSize.z; z++)
                    rawCells.push_back(MacGridCell{MacGridCell::Face(glm::dvec3((x + 1) * cellD.x, (y + 0.5) * cellD.y, (z + 0.5) * cellD.z)),
                                                   MacGridCell::Face(glm::dvec3((x + 0.5) * cellD.x, (y + 1) * cellD.y, (z + 0.5) * cellD.z)),
                                                   MacGridCell::Face(glm::dvec3((x + 0.5) * cellD.x, (y + 0.5) * cellD.y, (z + 1) * cellD.z)),
                                                   glm::dvec3(x + 0.5, y + 0.5, z + 0.5) * cellD});
    }
    MacGrid(const MacGrid&) = delete;
    virtual ~MacGrid() = default;

    MacGridCell& getCellAt(const glm::dvec3& p) { return cell(glm::ivec3(p * cellDInv)); }

    // Reference: macGrid.h:40 / macGrid.cpp:142-181.  The 8 faces of each axis
    // whose trilinear weights at `p` can be non-zero: for axis a the position in
    // cell units is shifted by half a cell on the two other axes, truncated
    // toward zero, and moved one cell down along a (face a of cell i sits at
    // (i + 1) h).  Entries come in the reference's corner order
    // (+x+y+z, +y+z, +x+z, +x+y, +x, +z, +y, base); the faces are those of the
    // host mirror (downloaded on first access after a step).
    std::array<std::array<MacGridCell::FaceRef, 8>, 3> getFacesAround(const glm::dvec3& p) {
        const glm::dvec3 g = p * cellDInv;
        glm::ivec3 base[3];
        for (int a = 0; a < 3; a++) {
            const double s[3] = {a == 0 ? 0.0 : 0.5, a == 1 ? 0.0 : 0.5, a == 2 ? 0.0 : 0.5};
            base[a] = glm::ivec3((int)(g.x - s[0]), (int)(g.y - s[1]), (int)(g.z - s[2]));
            base[a][a] -= 1;
        }
        auto face = [&](int a, int k) -> MacGridCell::FaceRef {
            const glm::ivec3 o = corner(k);
            return MacGridCell::FaceRef{cell(base[a].x + o.x, base[a].y + o.y, base[a].z + o.z).faces[a]};
        };
        return {std::array<MacGridCell::FaceRef, 8>{face(0, 0), face(0, 1), face(0, 2), face(0, 3), face(0, 4),
                                                    face(0, 5), face(0, 6), face(0, 7)},
                std::array<MacGridCell::FaceRef, 8>{face(1, 0), face(1, 1), face(1, 2), face(1, 3), face(1, 4),
                                                    face(1, 5), face(1, 6), face(1, 7)},
                std::array<MacGridCell::FaceRef, 8>{face(2, 0), face(2, 1), face(2, 2), face(2, 3), face(2, 4),
                                                    face(2, 5), face(2, 6), face(2, 7)}};
    }

    // Reference: macGrid.h:56 / macGrid.cpp:188-202.  The 8 cells whose centres
    // surround `p` (position in cell units minus one half, truncated toward
    // zero), in the same corner order as getFacesAround.  The manager's gfx fill
    // reads avgPNum through it (simulationManager.cpp:226-228).
    std::array<MacGridCellRef, 8> getCellsAround(const glm::dvec3& p) {
        const glm::dvec3 g = p * cellDInv;
        const glm::ivec3 b((int)(g.x - 0.5), (int)(g.y - 0.5), (int)(g.z - 0.5));
        auto at = [&](int k) -> MacGridCellRef {
            const glm::ivec3 o = corner(k);
            return MacGridCellRef{cell(b.x + o.x, b.y + o.y, b.z + o.z)};
        };
        return {at(0), at(1), at(2), at(3), at(4), at(5), at(6), at(7)};
    }

    template <int axis = 0, int offset = 0>
    MacGridCell& cell(const glm::ivec3& p) {
        pull();
        if constexpr (axis == 0) return rawCells[(size_t)(p.x + offset) * gridSize.y * gridSize.z + p.y * gridSize.z + p.z];
        else if constexpr (axis == 1) return rawCells[(size_t)p.x * gridSize.y * gridSize.z + (p.y + offset) * gridSize.z + p.z];
        else return rawCells[(size_t)p.x * gridSize.y * gridSize.z + p.y * gridSize.z + p.z + offset];
    }

    bool isPosValid(const glm::ivec3& p) {
        return p.x >= 0 && p.x < gridSize.x && p.y >= 0 && p.y < gridSize.y && p.z >= 0 && p.z < gridSize.z;
    }

    MacGridCell& cell(int x, int y, int z) {
        pull();
        return rawCells[(size_t)x * gridSize.y * gridSize.z + y * gridSize.z + z];
    }

    void forEachCell(bool /*parallel*/, bool includeBorders, std::function<void(glm::ivec3, MacGridCell&)>&& lambda) {
        pull();
        const int b = includeBorders ? 0 : 1;
        for (int x = b; x < gridSize.x - b; x++)
            for (int y = b; y < gridSize.y - b; y++)
                for (int z = b; z < gridSize.z - b; z++) lambda(glm::ivec3(x, y, z), cell(x, y, z));
    }

    void forEachFluidCell(bool parallel, std::function<void(glm::ivec3, MacGridCell&)>&& lambda) {
        forEachCell(parallel, false, [&](glm::ivec3 p, MacGridCell& c) {
            if (c.type == MacGridCell::CellType::WATER) lambda(p, c);
        });
    }

    // Reference: macGrid.h:139-145
    std::pair<glm::dvec3, glm::dvec3> getMinMaxRect(const glm::dvec3& p, const glm::dvec3& size) {
        const glm::dvec3 center = p * cellDInv;
        const glm::dvec3 d = size * cellDInv * 0.5;
        const glm::ivec3 mn(std::max(std::round(center.x - d.x), 1.0), std::max(std::round(center.y - d.y), 1.0),
                            std::max(std::round(center.z - d.z), 1.0));
        const glm::ivec3 mx(std::min(std::round(center.x + d.x), gridSize.x - 1.0),
                            std::min(std::round(center.y + d.y), gridSize.y - 1.0),
                            std::min(std::round(center.z + d.z), gridSize.z - 1.0));
        return std::make_pair(glm::dvec3(mn.x, mn.y, mn.z) * cellD, glm::dvec3(mx.x, mx.y, mx.z) * cellD);
    }

    // The pressure solve runs inside Simulator::simulate on the GPU; this solves
    // the bound context's current state (FSIM_STAGE_SOLVE) and returns the
    // iteration count.
    virtual int solveIncompressibility(bool parallel, double dt) = 0;

    const glm::dvec3 cellD;
    const glm::dvec3 cellDInv;
    const glm::ivec3 gridSize;
    const glm::dvec3 dimensions;

    bool isTopOfContainerSolid = false;
    double pressureK = 2.0, averagePressure = 2.0;
    int incompressibilityMaxIterationCount = 80;
    bool pressureEnabled = true;
    double fluidDensity = 1.0;
    double residualTolerance = 1e-6;

    const bool twoD;

protected:
    friend class simulator::Simulator;

    // Offset of corner k of a stencil in the reference's order.
    static glm::ivec3 corner(int k) {
        static const int o[8][3] = {{1, 1, 1}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0},
                                    {1, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 0, 0}};
        return glm::ivec3(o[k][0], o[k][1], o[k][2]);
    }

    void pull() {
        if (!device || host_valid) return;
        const size_t n = rawCells.size();
        std::vector<uint8_t> flags(n);
        std::vector<float> f(n);
        facade_detail::check(fsim_get_grid(device, FSIM_F_FLAGS, flags.data(), FSIM_HOST), device, "fsim_get_grid");
        for (size_t i = 0; i < n; i++) rawCells[i].type = (MacGridCell::CellType)flags[i];
        const int fv[3] = {FSIM_F_VX, FSIM_F_VY, FSIM_F_VZ}, fv2[3] = {FSIM_F_V2X, FSIM_F_V2Y, FSIM_F_V2Z};
        for (int a = 0; a < 3; a++) {
            facade_detail::check(fsim_get_grid(device, fv[a], f.data(), FSIM_HOST), device, "fsim_get_grid");
            for (size_t i = 0; i < n; i++) rawCells[i].faces[a].v = f[i];
            facade_detail::check(fsim_get_grid(device, fv2[a], f.data(), FSIM_HOST), device, "fsim_get_grid");
            for (size_t i = 0; i < n; i++) rawCells[i].faces[a].v2 = f[i];
        }
        facade_detail::check(fsim_get_grid(device, FSIM_F_AVGPNUM, f.data(), FSIM_HOST), device, "fsim_get_grid");
        for (size_t i = 0; i < n; i++) rawCells[i].avgPNum = f[i];
        host_valid = true;
    }

    std::vector<MacGridCell> rawCells;
    double resolution;
    glm::dvec3 requestedDimensions;
    fsim_ctx* device = nullptr;
    bool host_valid = true;
    double last_dt = 0;
};

class BridsonSolverGrid : public MacGrid {
public:
    // Reference: bridsonSolverGrid.h:14 (cellD is the resolution, cells per unit length)
    BridsonSolverGrid(const glm::dvec3& dimensions, float cellD, bool twoD, double fluidDensity)
        : MacGrid(dimensions, cellD, twoD) {
        this->fluidDensity = fluidDensity;
    }

    int solveIncompressibility(bool /*parallel*/, double dt) override {
        if (!device) throw std::runtime_error("solveIncompressibility: the grid is not bound to a Simulator");
        fsim_step_stats st{};
        facade_detail::check(fsim_stage(device, FSIM_STAGE_SOLVE, dt, &st), device, "fsim_stage(SOLVE)");
        host_valid = false;
        return st.pcg_iterations;
    }
};

// Reference: basicMacGrid.h:7-17 -- the SOR solver, selected by the manager for
// SimulationConfig::GridSolverType::BASIC (simulationManager.cpp:16-19).
class BasicMacGrid : public MacGrid {
public:
    using MacGrid::MacGrid;

    int solveIncompressibility(bool /*parallel*/, double dt) override {
        if (!device) throw std::runtime_error("solveIncompressibility: the grid is not bound to a Simulator");
        fsim_step_stats st{};
        facade_detail::check(fsim_stage(device, FSIM_STAGE_SOLVE, dt, &st), device, "fsim_stage(SOLVE)");
        host_valid = false;
        return st.pcg_iterations;
    }
};

}  // namespace macgrid

// ---------------------------------------------------------------- simulator
namespace simulator {

class Simulator {
public:
    enum class P2G2PType { PIC, FLIP, APIC };

    struct SimulatorConfig {
        P2G2PType transferType = P2G2PType::FLIP;
        float flipRatio = 0.99;
        float gravity = 150.0;
        bool gravityEnabled = true, pushParticlesApartEnabled = true;
        bool pushApartEnabled = true;
        bool particleSpawningEnabled = false;
        bool particleDespawningEnabled = false;
        bool stopParticles = false;
    };

    Simulator(SimulatorConfig config, std::shared_ptr<particles::HashedParticles> hashedParticles,
              std::shared_ptr<macgrid::MacGrid> macGrid)
        : config(std::move(config)), hashedParticles(std::move(hashedParticles)), macGrid(std::move(macGrid)) {
        for (const char* k : {"SimulateParticles", "PushParticlesApart", "PushParticlesOutOfObstacles", "P2GTransfer",
                              "IncompressibilityPrep", "Incompressibility", "VelocityExtrapolation", "G2PTransfer"})
            stepDuration[k] = 0;
    }
    Simulator(const Simulator&) = delete;
    ~Simulator() { release(); }

    void setNewMacGrid(std::shared_ptr<macgrid::MacGrid> grid) {
        release();
        macGrid = std::move(grid);
    }

    void setNewHashedParticles(std::shared_ptr<particles::HashedParticles> p) {
        if (hashedParticles) hashedParticles->pull();
        hashedParticles = std::move(p);
        if (hashedParticles) hashedParticles->edited = true;
    }

    // One Simulator::simulate(dt) (simulator.cpp:51-100) as one fsim_step.
    void simulate(double dt) {
        bind();
        fsim_params p = params();
        facade_detail::check(fsim_set_params(ctx, &p), ctx, "fsim_set_params");
        particles::HashedParticles& hp = *hashedParticles;
        if (hp.edited || hp.device != ctx) {
            hp.pull();
            hp.push(ctx);
        }
        std::vector<fsim_obstacle> obs;
        std::vector<obstacle::SphericalParticleSource*> sources;
        for (auto& o : obstacles) obs.push_back(convert(o.get(), sources));
        facade_detail::check(fsim_set_obstacles(ctx, obs.data(), (int)obs.size()), ctx, "fsim_set_obstacles");
        fsim_step_stats st{};
        facade_detail::check(fsim_step(ctx, dt, &st), ctx, "fsim_step");
        if (!sources.empty()) {
            std::vector<fsim_obstacle> back(obs.size());
            int n = 0;
            facade_detail::check(fsim_get_obstacles(ctx, back.data(), (int)back.size(), &n), ctx, "fsim_get_obstacles");
            size_t k = 0;
            for (int i = 0; i < n && k < sources.size(); i++)
                if (back[i].type == FSIM_OBS_SOURCE) sources[k++]->lastSpawnFraction = back[i].last_spawn_fraction;
        }
        hp.host_valid = false;
        macGrid->host_valid = false;
        macGrid->last_dt = dt;
        // sliding averages in microseconds, as the reference (simulator.cpp:52-99)
        constexpr double f = 0.9;
        auto upd = [&](const char* key, double ms) {
            stepDuration[key] = (long long)(stepDuration[key] * f + ms * 1000.0 * (1.0 - f));
        };
        upd("SimulateParticles", st.ms_simulate_particles);
        upd("PushParticlesApart", st.ms_push_apart);
        upd("PushParticlesOutOfObstacles", st.ms_push_out);
        upd("P2GTransfer", st.ms_p2g);
        upd("IncompressibilityPrep", st.ms_prep);
        upd("Incompressibility", st.ms_solve);
        stepDuration["Incompressibility it count"] = st.pcg_iterations;
        upd("VelocityExtrapolation", st.ms_extrapolate);
        upd("G2PTransfer", st.ms_g2p);
        last = st;
    }

    std::vector<std::unique_ptr<obstacle::Obstacle>> obstacles;

    std::map<std::string, long long> getStepDuration() const { return stepDuration; }

    SimulatorConfig config;

    // Extension: statistics of the last step and the library context.
    const fsim_step_stats& lastStats() const { return last; }
    fsim_ctx* context() { return ctx; }

private:
    fsim_params params() const {
        const macgrid::MacGrid& g = *macGrid;
        fsim_params p{};
        p.transfer = (int)config.transferType;
        p.flip_ratio = config.flipRatio;
        p.gravity = config.gravity;
        p.gravity_enabled = config.gravityEnabled;
        p.push_apart_enabled = config.pushApartEnabled;
        p.spawning_enabled = config.particleSpawningEnabled;
        p.despawning_enabled = config.particleDespawningEnabled;
        p.stop_particles = config.stopParticles;
        p.top_solid = g.isTopOfContainerSolid;
        p.pressure_enabled = g.pressureEnabled;
        p.pressure_k = g.pressureK;
        p.average_pressure = g.averagePressure;
        p.max_iters = g.incompressibilityMaxIterationCount;
        p.fluid_density = g.fluidDensity;
        p.residual_tol = g.residualTolerance;
        p.tol_mode = FSIM_TOL_ABS_MAX;
        p.particle_r = hashedParticles->getParticleR();
        p.precision = FSIM_PREC_MIXED;
        p.warm_start = FSIM_WARM_ZERO;
        p.track_ids = 0;
        p.timing = 1;
        p.precond = FSIM_PRECOND_MG;
        p.grid_solver = dynamic_cast<const macgrid::BasicMacGrid*>(&g) ? FSIM_SOLVER_SOR : FSIM_SOLVER_PCG;
        return p;
    }

    void bind() {
        if (ctx) return;
        macgrid::MacGrid& g = *macGrid;
        fsim_grid_desc gd{};
        gd.dims[0] = g.requestedDimensions.x;
        gd.dims[1] = g.requestedDimensions.y;
        gd.dims[2] = g.requestedDimensions.z;
        gd.resolution = g.resolution;
        gd.two_d = g.twoD ? 1 : 0;
        fsim_params p = params();
        fsim_ctx* c = nullptr;
        const int rc = fsim_create(&gd, &p, &c);
        if (rc != FSIM_OK) {
            std::string msg = "fsim_create failed (" + std::to_string(rc) + ")";
            if (c) {
                msg += std::string(": ") + fsim_last_error(c);
                fsim_destroy(c);
            }
            throw std::runtime_error(msg);
        }
        ctx = c;
        g.device = ctx;
        g.host_valid = true;
    }

    void release() {
        if (!ctx) return;
        if (hashedParticles && hashedParticles->device == ctx) {
            hashedParticles->pull();
            hashedParticles->device = nullptr;
            hashedParticles->edited = true;
        }
        if (macGrid && macGrid->device == ctx) {
            macGrid->pull();
            macGrid->device = nullptr;
        }
        fsim_destroy(ctx);
        ctx = nullptr;
    }

    // dynamic_cast dispatch as the reference's Simulator (simulator.cpp:106-312)
    static fsim_obstacle convert(obstacle::Obstacle* o, std::vector<obstacle::SphericalParticleSource*>& sources) {
        using namespace obstacle;
        fsim_obstacle f{};
        for (int a = 0; a < 3; a++) {
            f.pos[a] = o->pos[a];
            f.prev_pos[a] = o->prevPos[a];
            f.speed[a] = o->speed[a];
        }
        if (auto* s = dynamic_cast<SphericalParticleSource*>(o)) {
            f.type = FSIM_OBS_SOURCE;
            f.r = s->r;
            f.spawn_rate = s->particleSpawnRate;
            f.spawn_speed = s->particleSpawnSpeed;
            f.last_spawn_fraction = s->lastSpawnFraction;
            sources.push_back(s);
        } else if (auto* k = dynamic_cast<SphericalParticleSink*>(o)) {
            f.type = FSIM_OBS_SINK;
            f.r = k->r;
        } else if (auto* sp = dynamic_cast<SphericalObstacle*>(o)) {
            f.type = FSIM_OBS_SPHERE;
            f.r = sp->r;
        } else if (auto* d = dynamic_cast<DiscParticleSource*>(o)) {
            f.type = FSIM_OBS_DISC_SOURCE;
            f.r = d->r;
            f.spawn_speed = d->particleSpawnSpeed;
        } else if (auto* bs = dynamic_cast<RectengularParticleSink*>(o)) {
            f.type = FSIM_OBS_BOX_SINK;
            for (int a = 0; a < 3; a++) f.size[a] = bs->size[a];
        } else if (auto* b = dynamic_cast<RectengularObstacle*>(o)) {
            f.type = FSIM_OBS_BOX;
            for (int a = 0; a < 3; a++) f.size[a] = b->size[a];
        } else {
            throw std::runtime_error("unknown obstacle type");
        }
        return f;
    }

    std::shared_ptr<particles::HashedParticles> hashedParticles;
    std::shared_ptr<macgrid::MacGrid> macGrid;
    std::map<std::string, long long> stepDuration;
    fsim_ctx* ctx = nullptr;
    fsim_step_stats last{};
};

}  // namespace simulator
}  // namespace genericfsim

// Reference: util/interpolation.h:7-35 (global namespace, as the reference
// declares them).  Trilinear tent weight of a node at `center` seen from `pos`,
// prod over axes of (1 - |d|) with d the offset in cell units, and its gradient
// with respect to `pos` (component a: -sign(d_a) times the other two factors,
// in 1 / length units; +1 where d_a = 0).
inline double trilinearInterpoll(const glm::dvec3& center, const glm::dvec3& pos, const glm::dvec3 invCellD) {
    const glm::dvec3 d = (pos - center) * invCellD;
    return (1.0 - std::fabs(d.x)) * (1.0 - std::fabs(d.y)) * (1.0 - std::fabs(d.z));
}

inline glm::dvec3 trilinearInterpollGradient(const glm::dvec3& center, const glm::dvec3& pos,
                                             const glm::dvec3 invCellD) {
    const glm::dvec3 d = (pos - center) * invCellD;
    const double wx = 1.0 - std::fabs(d.x), wy = 1.0 - std::fabs(d.y), wz = 1.0 - std::fabs(d.z);
    const double sx = d.x > 0.0 ? -1.0 : 1.0, sy = d.y > 0.0 ? -1.0 : 1.0, sz = d.z > 0.0 ? -1.0 : 1.0;
    return glm::dvec3(sx * wy * wz, sy * wx * wz, sz * wx * wy) * invCellD;
}
