// k_particles.cu -- particle-side kernels: advection with wall / obstacle
// collisions, sink deletion, push-out, cell keys with warp-aggregated counts,
// the counting sort by cell (scan + scatter), the permuting gather, spawning
// and the renderer hand-off.
#include "fsim_ctx.h"

namespace {

// isParticleInRectangle (simulator.cpp:127-132)
__device__ __forceinline__ bool in_rect(float px, float py, float pz, float pr, float rx, float ry,
                                        float rz, const float* size) {
    return fabsf(px - rx) < size[0] * 0.5f + pr && fabsf(py - ry) < size[1] * 0.5f + pr &&
           fabsf(pz - rz) < size[2] * 0.5f + pr;
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) {
    return v < lo ? lo : (hi < v ? hi : v);
}

// One thread per particle.  Stages selected by flags:
//  do_advect: Simulator::advectParticles (simulator.cpp:134-251) in FP32 --
//             Euler step with up to 200 analytic wall bounces (restitution 0.3),
//             sphere / box obstacle back-stepping in 0.0002 s steps, sinks.
//  do_push:   Simulator::pushParticlesOutOfObstacles (simulator.cpp:253-312).
//  do_stop:   config.stopParticles (simulator.cpp:71-74).
//  do_key:    cell key trunc(pos/h) (same truncation as MacGrid::cell(pos*cellDInv),
//             simulator.cpp:357-359) and its rank inside the cell.  Lanes with
//             equal keys are merged with __match_any_sync so each cell counter
//             takes one atomic per warp.
__global__ void __launch_bounds__(256) k_advect(const AdvectArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < a.n;
    uint32_t key = FSIM_DEAD_KEY;
    if (live) {
        float px = a.p.p[0][i], py = a.p.p[1][i], pz = a.p.p[2][i];
        float vx = a.p.v[0][i], vy = a.p.v[1][i], vz = a.p.v[2][i];
        bool dead = a.keep_dead && a.key[i] == FSIM_DEAD_KEY;
        if (a.do_advect && !dead) {
            const float dt = a.dt, pr = a.pr;
            float t = 0.f;
            int run = 0;
            const int maxRun = 200;
            while (run < maxRun) {
                run++;
                float minT = 1e6f;
                int minAxis = 0;
                {
                    const float pp[3] = {px, py, pz}, vv[3] = {vx, vy, vz};
#pragma unroll
                    for (int ax = 0; ax < 3; ax++) {
                        float comp = vv[ax], tmp = 1e6f;
                        if (comp > 1e-6f) tmp = (a.hi[ax] - pp[ax]) / comp;
                        else if (comp < -1e-6f) tmp = (pp[ax] - a.lo[ax]) / -comp;
                        if (tmp < minT) { minT = tmp; minAxis = ax; }
                    }
                }
                if (minT <= dt - t) {
                    px = px + vx * minT * 0.999f;
                    py = py + vy * minT * 0.999f;
                    pz = pz + vz * minT * 0.999f;
                    if (minAxis == 0) vx *= -0.3f; else if (minAxis == 1) vy *= -0.3f; else vz *= -0.3f;
                    t += 0.999f * minT;
                    continue;
                }
                bool collision = false;
                const float rem = dt - t;
                px = px + vx * rem;
                py = py + vy * rem;
                pz = pz + vz * rem;
                for (int k = 0; k < a.nobs; k++) {
                    const DevObstacle& o = a.obs[k];
                    const float ox = o.pos[0], oy = o.pos[1], oz = o.pos[2];
                    const float sx = o.speed[0], sy = o.speed[1], sz = o.speed[2];
                    if (o.type == FSIM_OBS_BOX_SINK) {
                        if (a.despawn && fabsf(px - ox) < o.size[0] * 0.5f &&
                            fabsf(py - oy) < o.size[1] * 0.5f && fabsf(pz - oz) < o.size[2] * 0.5f) {
                            dead = true;
                            collision = false;
                            break;
                        }
                        continue;
                    }
                    if (o.type == FSIM_OBS_SPHERE || o.type == FSIM_OBS_SOURCE ||
                        o.type == FSIM_OBS_SINK) {
                        const float r = o.r + pr;
                        const float dx = ox - px, dy = oy - py, dz = oz - pz;
                        const float d = sqrtf(dx * dx + dy * dy + dz * dz) - r;
                        if (d < 0.f) {
                            if (o.type == FSIM_OBS_SINK && a.despawn) {
                                dead = true;
                                collision = false;
                                break;
                            }
                            float bt = 0.f;
                            for (;;) {
                                float ex = (px - vx * bt) - (ox - sx * bt);
                                float ey = (py - vy * bt) - (oy - sy * bt);
                                float ez = (pz - vz * bt) - (oz - sz * bt);
                                if (!(sqrtf(ex * ex + ey * ey + ez * ez) < r && bt < t + 0.001f)) break;
                                bt += 0.0002f;
                            }
                            if (bt > dt - t) continue;
                            bt += 0.0002f;
                            px -= bt * vx;
                            py -= bt * vy;
                            pz -= bt * vz;
                            const float tx = ox - sx * bt, ty = oy - sy * bt, tz = oz - sz * bt;
                            float nx = px - tx, ny = py - ty, nz = pz - tz;
                            const float inv = 1.f / sqrtf(nx * nx + ny * ny + nz * nz);
                            nx *= inv; ny *= inv; nz *= inv;
                            const float rvx = vx - sx, rvy = vy - sy, rvz = vz - sz;
                            const float semi = -(nx * rvx + ny * rvy + nz * rvz);
                            if (semi <= 0.f) continue;
                            const float mx = -rvx / semi, my = -rvy / semi, mz = -rvz / semi;
                            vx = ((nx - mx) * 2.f + mx) * semi + sx;
                            vy = ((ny - my) * 2.f + my) * semi + sy;
                            vz = ((nz - mz) * 2.f + mz) * semi + sz;
                            t += (dt - t) - bt;
                            collision = true;
                            break;
                        }
                    }
                    if (o.type == FSIM_OBS_BOX) {
                        if (in_rect(px, py, pz, pr, ox, oy, oz, o.size)) {
                            float bt = 0.f;
                            while (in_rect(px - vx * bt, py - vy * bt, pz - vz * bt, pr, ox - sx * bt,
                                           oy - sy * bt, oz - sz * bt, o.size) &&
                                   bt < dt - t)
                                bt += 0.0002f;
                            if (bt > dt - t) continue;
                            bt += 0.0002f;
                            px -= bt * vx;
                            py -= bt * vy;
                            pz -= bt * vz;
                            const float tp[3] = {ox - sx * bt, oy - sy * bt, oz - sz * bt};
                            float pp[3] = {px, py, pz}, vv[3] = {vx, vy, vz};
                            const float ss[3] = {sx, sy, sz};
                            for (int ax = 0; ax < 3; ax++) {
                                if (pp[ax] >= tp[ax] + o.size[ax] * 0.5f + pr) {
                                    vv[ax] = -vv[ax] * 0.2f + ss[ax];
                                    break;
                                } else if (pp[ax] <= tp[ax] - o.size[ax] * 0.5f - pr) {
                                    vv[ax] = -vv[ax] * 0.2f - ss[ax];
                                    break;
                                }
                            }
                            vx = vv[0]; vy = vv[1]; vz = vv[2];
                            t += (dt - t) - bt;
                            collision = true;
                            break;
                        }
                    }
                }
                if (!collision) run = maxRun;
            }
            px = clampf(px, a.lo[0], a.hi[0]);
            py = clampf(py, a.lo[1], a.hi[1]);
            pz = clampf(pz, a.lo[2], a.hi[2]);
        }
        if (a.do_push && !dead) {
            for (int k = 0; k < a.nobs; k++) {
                const DevObstacle& o = a.obs[k];
                if (o.type == FSIM_OBS_SPHERE || o.type == FSIM_OBS_SOURCE || o.type == FSIM_OBS_SINK) {
                    const float r = o.r + a.pr;
                    const float dx = px - o.pos[0], dy = py - o.pos[1], dz = pz - o.pos[2];
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 < r * r) {
                        const float dist = sqrtf(d2);
                        px = clampf(o.pos[0] + dx / dist * r, a.plo[0], a.phi[0]);
                        py = clampf(o.pos[1] + dy / dist * r, a.plo[1], a.phi[1]);
                        // zConst (simulator.cpp:276): 2D particles go back to the plane
                        pz = a.g.two_d ? a.g.zc : clampf(o.pos[2] + dz / dist * r, a.plo[2], a.phi[2]);
                    }
                } else if (o.type == FSIM_OBS_BOX) {
                    // in 2D the z extent is not tested and z is never the push axis
                    // (simulator.cpp:285-290)
                    if (!(px > o.box_hi[0] || px < o.box_lo[0] || py > o.box_hi[1] || py < o.box_lo[1] ||
                          ((pz > o.box_hi[2] || pz < o.box_lo[2]) && !a.g.two_d))) {
                        float pp[3] = {px, py, pz};
                        int axis = 0;
                        float amount = 1e6f;
                        const int naxes = a.g.two_d ? 2 : 3;
                        for (int q = 0; q < naxes; q++) {
                            if (pp[q] > o.pos[q]) {
                                float tmp = o.box_hi[q] - pp[q];
                                if (tmp < fabsf(amount)) { amount = tmp; axis = q; }
                            } else {
                                float tmp = o.box_lo[q] - pp[q];
                                if (-tmp < fabsf(amount)) { amount = tmp; axis = q; }
                            }
                        }
                        pp[axis] = clampf(pp[axis] + amount, a.plo[axis], a.phi[axis]);
                        px = pp[0]; py = pp[1]; pz = pp[2];
                    }
                }
            }
        }
        if (a.do_stop) { vx = 0.f; vy = 0.f; vz = 0.f; }
        if (dead && a.keep_dead) {
            // deleted by the first pass: nothing moves
        } else if (a.do_advect || a.do_push) {
            a.p.p[0][i] = px; a.p.p[1][i] = py; a.p.p[2][i] = pz;
        }
        if (a.do_advect || a.do_stop) {
            a.p.v[0][i] = vx; a.p.v[1][i] = vy; a.p.v[2][i] = vz;
        }
        if (a.do_key && !dead) {
            int cx = (int)(px * a.g.hinv), cy = (int)(py * a.g.hinv), cz = (int)(pz * a.g.hzinv);
            cx = min(max(cx, 0), a.g.nx - 1);
            cy = min(max(cy, 0), a.g.ny - 1);
            cz = min(max(cz, 0), a.g.nz - 1);
            key = (uint32_t)gidx(a.g, cx, cy, cz);
        }
    }
    if (!a.do_key) return;
    // warp-aggregated cell counting: one atomic per distinct key per warp
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (key != FSIM_DEAD_KEY && lane == leader) base = (unsigned)atomicAdd(&a.count[key], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (live) {
        a.key[i] = key;
        a.rank[i] = base + __popc(peers & ((1u << lane) - 1u));
    }
}

// ---- exclusive scan (three kernels: tile sums, scan of sums, tile scan) ----
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int block_excl_scan(int v, int* total) {
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    int excl = x - v + (warp > 0 ? warp_sums[warp - 1] : 0);
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_tile_sums(const int* in, long long n, int* sums) {
    const long long base = (long long)blockIdx.x * SCAN_TILE;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        long long j = base + (long long)k * SCAN_THREADS + threadIdx.x;
        if (j < n) s += in[j];
    }
    __shared__ int red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int t = red[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = t;
    }
}

// single block: exclusive scan of the tile sums in place (any count)
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(int* sums, int nt) {
    int carry = 0;
    for (int base = 0; base < nt; base += SCAN_THREADS) {
        int j = base + threadIdx.x;
        int v = j < nt ? sums[j] : 0;
        int total;
        int e = block_excl_scan(v, &total);
        if (j < nt) sums[j] = e + carry;
        carry += total;
    }
}

// out[j] = exclusive prefix of in, out[n] = total
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_scan(const int* in, long long n, const int* sums,
                                                            int* out) {
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        local += v[k];
    }
    int total;
    int e = block_excl_scan(local, &total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = e;
        e += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = e;
}

// HashedParticles::pushParticlesApart (hashedParticles.cpp:64-107) with
// deterministic (Jacobi) semantics: every particle moves by the sum, over all
// other particles within distance 2r (and not closer than 1e-4), of half the
// overlap along their separation, computed from the positions at the start of
// the pass, then is clamped to [h + 1.01 r, dims - h - 1.01 r].  (The
// reference updates both particles of a pair in place, in a racy parallel
// loop; for an isolated pair both give the same result.)  Neighbours come from
// the cell sort: with 2r <= h they lie in the 27 cells around the particle's
// cell.  New positions go to out; thread = sorted slot.
__global__ void k_push_apart(ParticleBuf p, const uint32_t* perm, const int* cstart, GridGeom g, long long n,
                             float r, float lo0, float lo1, float lo2, float hi0, float hi1, float hi2,
                             float* out0, float* out1, float* out2) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long live = cstart[g.ncell];
    if (k >= live || k >= n) return;
    const uint32_t i = perm[k];
    const float xi = p.p[0][i], yi = p.p[1][i], zi = p.p[2][i];
    const int cx = (int)(xi * g.hinv), cy = (int)(yi * g.hinv), cz = (int)(zi * g.hzinv);
    const float D = 2.f * r, D2 = D * D;
    float dx = 0.f, dy = 0.f, dz = 0.f;
    for (int ox = -1; ox <= 1; ox++) {
        const int x = cx + ox;
        if (x < 0 || x >= g.nx) continue;
        for (int oy = -1; oy <= 1; oy++) {
            const int y = cy + oy;
            if (y < 0 || y >= g.ny) continue;
            // the three z cells of a row are one contiguous run of the sort
            const int zb = max(cz - 1, 0), ze = min(cz + 2, g.nz);
            const long long row = gidx(g, x, y, 0);
            const int b = cstart[row + zb], e = cstart[row + ze];
            for (int q = b; q < e; q++) {
                const uint32_t j = perm[q];
                if (j == i) continue;
                const float px = xi - p.p[0][j], py = yi - p.p[1][j], pz = zi - p.p[2][j];
                const float d2 = px * px + py * py + pz * pz;
                if (d2 > D2 || d2 < 1e-8f) continue;
                const float d = sqrtf(d2);
                const float t = (D - d) / d * 0.5f;
                dx += px * t;
                dy += py * t;
                dz += pz * t;
            }
        }
    }
    out0[i] = fminf(fmaxf(xi + dx, lo0), hi0);
    out1[i] = fminf(fmaxf(yi + dy, lo1), hi1);
    out2[i] = g.two_d ? g.zc : fminf(fmaxf(zi + dz, lo2), hi2);  // zConst (hashedParticles.cpp:98)
}

__global__ void k_scatter(const uint32_t* key, const uint32_t* rank, const int* cstart, uint32_t* perm,
                          long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = key[i];
    if (k == FSIM_DEAD_KEY) return;
    perm[cstart[k] + rank[i]] = (uint32_t)i;
}

// Stable cell order: the scatter places a cell's particles in the order their
// warps won the count atomics, which varies from run to run.  This pass sorts
// every cell's segment of perm by particle index, so the order inside a cell is
// the order of the particle buffer (itself the previous step's cell order) and
// every later sum over a cell's particles is reproducible.  Segments are
// usually in order already (a cell's particles mostly share a warp); the
// others of up to 16 entries go through a bitonic network in registers, longer
// ones through an insertion sort in place.
__device__ __forceinline__ void cswap(uint32_t& a, uint32_t& b, bool up) {
    const uint32_t lo = min(a, b), hi = max(a, b);
    a = up ? lo : hi;
    b = up ? hi : lo;
}

__global__ void k_cell_order(uint32_t* perm, const int* cstart, long long ncell) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int beg = cstart[c], end = cstart[c + 1];
    const int len = end - beg;
    if (len < 2) return;
    bool sorted = true;
    uint32_t prev = perm[beg];
    for (int k = beg + 1; k < end; k++) {
        const uint32_t x = perm[k];
        sorted &= prev < x;
        prev = x;
    }
    if (sorted) return;
    if (len <= 16) {
        uint32_t v[16];
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = k < len ? perm[beg + k] : 0xFFFFFFFFu;
#pragma unroll
        for (int size = 2; size <= 16; size <<= 1)
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1)
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int l = k ^ stride;
                    if (l > k) cswap(v[k], v[l], (k & size) == 0);
                }
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (k < len) perm[beg + k] = v[k];
        return;
    }
    for (int k = beg + 1; k < end; k++) {
        const uint32_t x = perm[k];
        int j = k - 1;
        while (j >= beg && perm[j] > x) {
            perm[j + 1] = perm[j];
            j--;
        }
        perm[j + 1] = x;
    }
}

// dst[j] = src[perm[j]] for the j < cstart[ncell] live particles
__global__ void k_gather(ParticleBuf src, ParticleBuf dst, const uint32_t* perm, const int* cstart,
                         long long ncell, long long n, int ids) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = cstart[ncell];
    if (j >= n || j >= total) return;
    const uint32_t i = perm[j];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        dst.p[a][j] = src.p[a][i];
        dst.v[a][j] = src.v[a][i];
    }
#pragma unroll
    for (int a = 0; a < 9; a++) dst.c[a][j] = src.c[a][i];
    if (ids) dst.id[j] = src.id[i];
}

// SphericalParticleSource emission (simulator.cpp:106-125): positions on the
// sphere of radius r_src + r_particle at angles theta in [0, 2pi), phi in [0, pi)
// (the reference's distribution), velocity along the outward normal.  Angles
// come from SplitMix64 draws instead of the C library's rand().
__global__ void k_spawn_sphere(ParticleBuf p, long long first, int count, double ox, double oy,
                               double oz, double r, double speed, uint64_t seed, uint32_t first_id,
                               int ids) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const double kPi = 3.14159265358979323846;
    const double theta = 2.0 * kPi * uniform01(seed, 2ull * k);
    const double phi = kPi * uniform01(seed, 2ull * k + 1);
    const double nx = r * sin(phi) * cos(theta), ny = r * sin(phi) * sin(theta), nz = r * cos(phi);
    const double inv = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
    const long long i = first + k;
    p.p[0][i] = (float)(ox + nx);
    p.p[1][i] = (float)(oy + ny);
    p.p[2][i] = (float)(oz + nz);
    p.v[0][i] = (float)(speed * (nx * inv));
    p.v[1][i] = (float)(speed * (ny * inv));
    p.v[2][i] = (float)(speed * (nz * inv));
#pragma unroll
    for (int a = 0; a < 9; a++) p.c[a][i] = 0.f;
    if (ids) p.id[i] = first_id + (uint32_t)k;
}

// Disc source (extension): 8 particles per covered cell, one per 2x2x2
// sub-cell with +-0.5 sub-cell jitter, velocity (0, speed, 0).  In 2D mode the
// particles sit on the plane z = zc.
__global__ void k_spawn_disc(ParticleBuf p, long long first, int ncells, const int* cells_xz, int cy,
                             GridGeom g, float vy, uint64_t seed, uint32_t first_id, int ids) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncells * 8) return;
    const int c = k >> 3, s = k & 7;
    const int cx = cells_xz[2 * c], cz = cells_xz[2 * c + 1];
    const double sub[3] = {(s & 4) ? 0.75 : 0.25, (s & 2) ? 0.75 : 0.25, (s & 1) ? 0.75 : 0.25};
    const double base[3] = {(double)cx, (double)cy, (double)cz};
    const long long i = first + k;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double u = uniform01(seed, 3ull * k + a);
        p.p[a][i] = (float)((base[a] + sub[a] + (u - 0.5) * 0.5 * 0.999) * (a == 2 ? g.hzd : g.hd));
    }
    if (g.two_d) p.p[2][i] = g.zc;
    p.v[0][i] = 0.f;
    p.v[1][i] = vy;
    p.v[2][i] = 0.f;
#pragma unroll
    for (int a = 0; a < 9; a++) p.c[a][i] = 0.f;
    if (ids) p.id[i] = first_id + (uint32_t)k;
}

// SimulationManager gfx publish (simulationManager.cpp:218-231): position,
// |v| and the trilinear interpolation of avgPNum at the particle.
constexpr int GFX_THREADS = 256;

// One 20-byte record per particle.  vec (out 16-byte aligned): the block's
// records are staged in shared memory and written as contiguous 16-byte
// stores (a block's records start at 256 * 20 bytes, a multiple of 16), not
// as five 4-byte stores at a 20-byte stride per lane.
__global__ void __launch_bounds__(GFX_THREADS) k_gfx(ParticleBuf p, long long n, const float* avg, GridGeom g,
                                                     fsim_particle_gfx* out, int vec) {
    __shared__ __align__(16) float stage[GFX_THREADS * 5];
    const long long i0 = (long long)blockIdx.x * GFX_THREADS;
    const long long i = i0 + threadIdx.x;
    float rec[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (i < n) {
        const float px = p.p[0][i], py = p.p[1][i], pz = p.p[2][i];
        const float vx = p.v[0][i], vy = p.v[1][i], vz = p.v[2][i];
        const float gx = px * g.hinv - 0.5f, gy = py * g.hinv - 0.5f, gz = pz * g.hzinv - 0.5f;
        const int bx = (int)gx, by = (int)gy, bz = (int)gz;
        float dens = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int x = bx + (k >> 2), y = by + ((k >> 1) & 1), z = bz + (k & 1);
            if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) continue;
            const float w = (1.f - fabsf(gx - x)) * (1.f - fabsf(gy - y)) * (1.f - fabsf(gz - z));
            dens += w * avg[gidx(g, x, y, z)];
        }
        rec[0] = px;
        rec[1] = py;
        rec[2] = pz;
        rec[3] = sqrtf(vx * vx + vy * vy + vz * vz);
        rec[4] = dens;
    }
    if (!vec) {
        if (i < n) {
            fsim_particle_gfx o;
            o.pos[0] = rec[0]; o.pos[1] = rec[1]; o.pos[2] = rec[2];
            o.v = rec[3];
            o.density = rec[4];
            out[i] = o;
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < 5; k++) stage[threadIdx.x * 5 + k] = rec[k];
    __syncthreads();
    const long long nrec = n - i0 < GFX_THREADS ? n - i0 : GFX_THREADS;
    const int nfl = (int)(nrec * 5), nf4 = nfl >> 2;
    float* dst = reinterpret_cast<float*>(out) + i0 * 5;
    for (int q = threadIdx.x; q < nf4; q += GFX_THREADS)
        reinterpret_cast<float4*>(dst)[q] = reinterpret_cast<const float4*>(stage)[q];
    if ((int)threadIdx.x < nfl - 4 * nf4) dst[4 * nf4 + threadIdx.x] = stage[4 * nf4 + threadIdx.x];
}

}  // namespace

void launch_advect(const AdvectArgs& a, cudaStream_t s) {
    if (a.n <= 0) return;
    k_advect<<<ceil_div(a.n, 256), 256, 0, s>>>(a);
}

void launch_scan(const int* in, int* out, long long n, int* block_sums, cudaStream_t s) {
    const int nt = ceil_div(n, SCAN_TILE);
    k_tile_sums<<<nt, SCAN_THREADS, 0, s>>>(in, n, block_sums);
    k_scan_sums<<<1, SCAN_THREADS, 0, s>>>(block_sums, nt);
    k_tile_scan<<<nt, SCAN_THREADS, 0, s>>>(in, n, block_sums, out);
}

void launch_push_apart(ParticleBuf p, const uint32_t* perm, const int* cstart, const GridGeom& g, long long n,
                       double r, const float lo[3], const float hi[3], float* const out[3], cudaStream_t s) {
    if (n <= 0) return;
    k_push_apart<<<ceil_div(n, 256), 256, 0, s>>>(p, perm, cstart, g, n, (float)r, lo[0], lo[1], lo[2], hi[0], hi[1],
                                                  hi[2], out[0], out[1], out[2]);
}

void launch_scatter(const uint32_t* key, const uint32_t* rank, const int* cstart, uint32_t* perm,
                    long long n, long long ncell, cudaStream_t s) {
    if (n <= 0) return;
    k_scatter<<<ceil_div(n, 256), 256, 0, s>>>(key, rank, cstart, perm, n);
    k_cell_order<<<ceil_div(ncell, 256), 256, 0, s>>>(perm, cstart, ncell);
}

void launch_gather(ParticleBuf src, ParticleBuf dst, const uint32_t* perm, const int* cstart,
                   long long ncell, long long n, bool ids, cudaStream_t s) {
    if (n <= 0) return;
    k_gather<<<ceil_div(n, 256), 256, 0, s>>>(src, dst, perm, cstart, ncell, n, ids ? 1 : 0);
}

void launch_spawn_sphere(ParticleBuf p, long long first, int count, const fsim_obstacle& o,
                         double particle_r, uint64_t seed, uint32_t first_id, bool ids,
                         cudaStream_t s) {
    if (count <= 0) return;
    k_spawn_sphere<<<ceil_div(count, 128), 128, 0, s>>>(p, first, count, o.pos[0], o.pos[1], o.pos[2],
                                                        o.r + particle_r, o.spawn_speed, seed, first_id,
                                                        ids ? 1 : 0);
}

void launch_spawn_disc(ParticleBuf p, long long first, int ncells, const fsim_obstacle& o,
                       const GridGeom& g, int cy, const int* cells_xz, uint64_t seed,
                       uint32_t first_id, bool ids, cudaStream_t s) {
    if (ncells <= 0) return;
    k_spawn_disc<<<ceil_div(ncells * 8, 128), 128, 0, s>>>(p, first, ncells, cells_xz, cy, g,
                                                           (float)o.spawn_speed, seed, first_id,
                                                           ids ? 1 : 0);
}

void launch_gfx(ParticleBuf p, long long n, const float* avg, const GridGeom& g,
                fsim_particle_gfx* out, cudaStream_t s) {
    if (n <= 0) return;
    const int vec = (reinterpret_cast<uintptr_t>(out) & 15) == 0 ? 1 : 0;
    k_gfx<<<ceil_div(n, GFX_THREADS), GFX_THREADS, 0, s>>>(p, n, avg, g, out, vec);
}
