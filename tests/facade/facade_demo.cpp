// Drives the GPU library through the reference-shaped C++ facade the way the
// reference's SimulationManager does (simulationManager.cpp:10-29,170-245):
// build a BridsonSolverGrid, a HashedParticles and a Simulator, set the
// obstacles, call simulate(dt) K times, read the particles back through
// getParticleAt.  Input / output: raw float32 arrays (pos n x 3).
//
//   facade_demo <resolution> <steps> <dt> <transfer 0|1|2> <in_pos.bin> <out.bin> [basic|2d]
//
// With "basic", the grid is a BasicMacGrid (the SOR solver); with "2d" the
// grid and the particles are built in 2D mode (dims (1, 1, 0.3), particles on
// z = 0.15), as SimulationManager does for twoD (simulationManager.cpp:17,27).
//
// out.bin: int64 n, then pos (n x 3), v (n x 3), c (n x 9) as float32, then
// int32 PCG iterations of the last step, then the renderer's per-particle
// density (n float32) computed as SimulationManager's gfx fill does it
// (simulationManager.cpp:222-230: getCellsAround + trilinearInterpoll of
// avgPNum).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <iostream>
#include <vector>

#include "fsim_facade.hpp"

using namespace genericfsim;

int main(int argc, char** argv) {
    if (argc != 7 && argc != 8) {
        std::cerr << "usage: facade_demo res steps dt transfer in_pos.bin out.bin [basic|2d]\n";
        return 2;
    }
    const bool basic = argc == 8 && std::string(argv[7]) == "basic";
    const bool two_d = argc == 8 && std::string(argv[7]) == "2d";
    const glm::dvec3 dims = two_d ? glm::dvec3(1, 1, 0.3) : glm::dvec3(1, 1, 1);
    const double zc = two_d ? 0.15 : 0.5;
    const double res = std::atof(argv[1]);
    const int steps = std::atoi(argv[2]);
    const double dt = std::atof(argv[3]);
    const int transfer = std::atoi(argv[4]);
    std::ifstream in(argv[5], std::ios::binary | std::ios::ate);
    const std::streamsize bytes = in.tellg();
    in.seekg(0);
    std::vector<float> pos((size_t)bytes / 4);
    in.read(reinterpret_cast<char*>(pos.data()), bytes);
    const size_t n = pos.size() / 3;
    try {
        std::shared_ptr<macgrid::MacGrid> grid;
        if (basic) grid = std::make_shared<macgrid::BasicMacGrid>(dims, res, two_d);
        else grid = std::make_shared<macgrid::BridsonSolverGrid>(dims, (float)res, two_d, 1.0);
        grid->isTopOfContainerSolid = true;
        grid->pressureEnabled = false;
        grid->incompressibilityMaxIterationCount = 200;
        grid->residualTolerance = 1e-6;
        const double h = 1.0 / res;
        auto parts = std::make_shared<particles::HashedParticles>(0, h / 4, grid->dimensions, grid->cellD, two_d,
                                                                  dims.z / 2);
        std::vector<particles::Particle> ps(n);
        for (size_t i = 0; i < n; i++) {
            ps[i].pos = glm::dvec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
            ps[i].v = glm::dvec3(0, 0, 0);
            ps[i].c[0] = ps[i].c[1] = ps[i].c[2] = glm::dvec3(0, 0, 0);
        }
        parts->addParticles(std::move(ps));
        simulator::Simulator::SimulatorConfig cfg;
        cfg.transferType = (simulator::Simulator::P2G2PType)transfer;
        cfg.flipRatio = 0.95f;
        cfg.gravity = -9.81f;
        cfg.pushApartEnabled = false;
        simulator::Simulator sim(cfg, parts, grid);
        sim.obstacles.push_back(std::make_unique<obstacle::SphericalObstacle>(0.15, glm::dvec3(0.6, 0.3, zc)));
        for (int s = 0; s < steps; s++) {
            sim.obstacles[0]->setNewPos(glm::dvec3(0.6 + 0.01 * s, 0.3, zc));
            sim.obstacles[0]->calculateSpeed(dt);
            sim.simulate(dt);
        }
        const auto dur = sim.getStepDuration();
        const int its = (int)dur.at("Incompressibility it count");
        const int m = parts->getParticleNum();
        std::vector<float> p3((size_t)m * 3), v3((size_t)m * 3), c9((size_t)m * 9);
        for (int i = 0; i < m; i++) {
            const particles::Particle& q = parts->getParticleAt(i);
            for (int a = 0; a < 3; a++) {
                p3[3 * i + a] = (float)q.pos[a];
                v3[3 * i + a] = (float)q.v[a];
                for (int b = 0; b < 3; b++) c9[9 * i + 3 * a + b] = (float)q.c[a][b];
            }
        }
        // ParticleGfxData::density, as the manager's gfx fill computes it
        std::vector<float> dens((size_t)m);
        parts->forEach(true, [&](particles::Particle& q, int index) {
            float density = 0;
            auto cells = grid->getCellsAround(q.pos);
            for (auto& c : cells) density += trilinearInterpoll(q.pos, c.cell.pos, grid->cellDInv) * c.cell.avgPNum;
            dens[(size_t)index] = density;
        });
        // the stencils are partitions of unity: for every particle the tent
        // weights of the 8 faces of each axis (getFacesAround) and of the 8 cell
        // centres (getCellsAround) are non-negative and sum to 1
        for (int i = 0; i < m && !two_d; i++) {
            const glm::dvec3 q = parts->getParticleAt(i).pos;
            const auto faces = grid->getFacesAround(q);
            const auto cells = grid->getCellsAround(q);
            for (int a = 0; a < 4; a++) {
                double sum = 0, lo = 1;
                for (int k = 0; k < 8; k++) {
                    const glm::dvec3 node = a < 3 ? faces[a][k].face.pos : cells[k].cell.pos;
                    const double w = trilinearInterpoll(node, q, grid->cellDInv);
                    sum += w;
                    lo = std::min(lo, w);
                }
                if (std::fabs(sum - 1.0) > 1e-9 || lo < -1e-9) {
                    std::cerr << "stencil " << a << " of particle " << i << ": weight sum " << sum << "\n";
                    return 3;
                }
            }
        }
        // a cell read through the grid mirror, as SimulationManager::getCellAt does
        const macgrid::MacGridCell& cell = grid->getCellAt(glm::dvec3(0.3, 0.1, zc));
        std::ofstream out(argv[6], std::ios::binary);
        const int64_t mm = m;
        out.write(reinterpret_cast<const char*>(&mm), 8);
        out.write(reinterpret_cast<const char*>(p3.data()), p3.size() * 4);
        out.write(reinterpret_cast<const char*>(v3.data()), v3.size() * 4);
        out.write(reinterpret_cast<const char*>(c9.data()), c9.size() * 4);
        out.write(reinterpret_cast<const char*>(&its), 4);
        out.write(reinterpret_cast<const char*>(dens.data()), dens.size() * 4);
        std::cout << "particles " << m << " its " << its << " cell_type " << (int)cell.type << "\n";
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
