// k_grid.cu -- grid-side kernels: obstacle rasterisation, container walls,
// v2 = v + gravity, velocity extrapolation, pressure application, and the
// conversions between the padded device layout and the reference cell order.
#include <cmath>

#include "fsim_ctx.h"

namespace {

__device__ __forceinline__ bool in_grid(const GridGeom& g, int x, int y, int z) {
    return x >= 0 && y >= 0 && z >= 0 && x < g.nx && y < g.ny && z < g.nz;
}

// ---- obstacles (MacGrid::addObstacle, macGrid.cpp:231-292) -----------------
//
// The reference walks the obstacle's cells serially in x, y, z order, turning
// each covered cell SOLID and setting the normal velocity of every face it
// shares with a WATER cell to the obstacle speed.  Because the +x/+y/+z
// neighbours of a cell are visited after it, the serial result is reproduced in
// parallel: for the face between cells A (low side) and B = A + e_a, with T0
// the cell types before this obstacle,
//     v = speed_a   if (A covered and T0(B) == WATER)
//                   or (B covered and A not covered and T0(A) == WATER).
// Kernel 1 applies that to faces (reading only T0), kernel 2 marks the covered
// cells SOLID.  The coverage tests are evaluated in FP64 exactly as the
// reference does.
struct ObsGeom {
    int kind;               // 0 sphere (incl. source), 1 box
    double cx, cy, cz, r2;  // sphere: centre and squared radius in cell units
    int mn[3], mx[3];       // covered index range: sphere inclusive, box exclusive upper
    float speed[3];
};

__device__ __forceinline__ bool covered(const ObsGeom& o, int x, int y, int z) {
    if (o.kind == 0) {
        if (x < o.mn[0] || x > o.mx[0] || y < o.mn[1] || y > o.mx[1] || z < o.mn[2] || z > o.mx[2])
            return false;
        const double dx = (x + 0.5) - o.cx, dy = (y + 0.5) - o.cy, dz = (z + 0.5) - o.cz;
        return dx * dx + dy * dy + dz * dz < o.r2;
    }
    return x >= o.mn[0] && x < o.mx[0] && y >= o.mn[1] && y < o.mx[1] && z >= o.mn[2] && z < o.mx[2];
}

// threads over the covered index box extended by one cell on the low side
__global__ void k_obstacle_faces(GridGeom g, ObsGeom o, const uint8_t* flags, float* u0, float* u1,
                                 float* u2, int ex, int ey, int ez) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ex * ey * ez) return;
    const int x = o.mn[0] - 1 + t / (ey * ez), y = o.mn[1] - 1 + (t / ez) % ey, z = o.mn[2] - 1 + t % ez;
    if (!in_grid(g, x, y, z)) return;
    const bool ca = covered(o, x, y, z);
    const uint8_t ta = flags[gidx(g, x, y, z)];
    float* u[3] = {u0, u1, u2};
    const int d[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int bx = x + d[a][0], by = y + d[a][1], bz = z + d[a][2];
        if (!in_grid(g, bx, by, bz)) continue;
        const bool cb = covered(o, bx, by, bz);
        const uint8_t tb = flags[gidx(g, bx, by, bz)];
        if ((ca && tb == C_WATER) || (cb && !ca && ta == C_WATER)) u[a][gidx(g, x, y, z)] = o.speed[a];
    }
}

__global__ void k_obstacle_cells(GridGeom g, ObsGeom o, uint8_t* flags, int ex, int ey, int ez) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ex * ey * ez) return;
    const int x = o.mn[0] + t / (ey * ez), y = o.mn[1] + (t / ez) % ey, z = o.mn[2] + t % ez;
    if (!in_grid(g, x, y, z)) return;
    if (covered(o, x, y, z)) flags[gidx(g, x, y, z)] = C_SOLID;
}

// ---- walls + v2 (restoreBorderingSolidCellsAndSpeeds, macGrid.cpp:75-140;
//      postP2GUpdate, macGrid.cpp:204-219) --------------------------------------
__device__ __forceinline__ bool is_border(const GridGeom& g, int top_solid, int x, int y, int z) {
    return x == 0 || x == g.nx - 1 || y == 0 || (top_solid && y == g.ny - 1) || z == 0 || z == g.nz - 1;
}

// One thread per cell.  walls: border cells become SOLID; the face between a
// border cell and a WATER cell gets v = 0.  post: v2 = v, plus the gravity
// increment on y-faces whose two cells are not SOLID (the cell "above" the top
// row counts as SOLID, as the reference's aliased index resolves to the floor).
__global__ void k_prep(GridGeom g, int top_solid, int walls, int post, float ginc, uint8_t* flags,
                       float* u0, float* u1, float* u2, float* w0, float* w1, float* w2) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    if (z >= g.nz) return;
    const bool bc = is_border(g, top_solid, x, y, z);
    uint8_t fc = flags[c];
    if (walls && bc) fc = C_SOLID;
    float uu[3] = {u0[c], u1[c], u2[c]};
    if (walls) {
        const long long st[3] = {(long long)g.pz * g.ny, g.pz, 1};
        const int pos[3] = {x, y, z}, lim[3] = {g.nx, g.ny, g.nz};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (pos[a] + 1 >= lim[a]) continue;
            const int nxp = x + (a == 0), nyp = y + (a == 1), nzp = z + (a == 2);
            const bool bn = is_border(g, top_solid, nxp, nyp, nzp);
            const uint8_t fn = bn ? (uint8_t)C_SOLID : flags[c + st[a]];
            if ((bc && fn == C_WATER) || (bn && fc == C_WATER)) uu[a] = 0.f;
        }
        if (bc) flags[c] = C_SOLID;
        u0[c] = uu[0];
        u1[c] = uu[1];
        u2[c] = uu[2];
    }
    if (post) {
        float vy = uu[1];
        if (fc != C_SOLID && y + 1 < g.ny) {
            const bool bn = walls ? is_border(g, top_solid, x, y + 1, z) : false;
            const uint8_t fn = bn ? (uint8_t)C_SOLID : flags[c + g.pz];
            if (fn != C_SOLID) vy += ginc;
        }
        w0[c] = uu[0];
        w1[c] = vy;
        w2[c] = uu[2];
    }
}

// ---- extrapolation (MacGrid::extrapolateVelocities, macGrid.cpp:294-336) ----
// valid = 0 on fluid cells, 100 elsewhere.  Pass it: every cell with
// valid > it averages the three face v2 values of each neighbour with
// valid <= it and writes its own face a when the +a neighbour is inside the grid
// and not WATER; it then gets valid = it + 1.  Cells written in a pass are never
// read as sources in that pass, so the passes are order independent.
__global__ void k_extrapolate(GridGeom g, int it, const uint8_t* flags, uint8_t* valid, float* v0,
                              float* v1, float* v2) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    if (z >= g.nz) return;
    auto vld = [&](long long cc) -> int {
        return it == 0 ? (flags[cc] == C_WATER ? 0 : 100) : valid[cc];
    };
    const int mine = vld(c);
    if (it == 0) valid[c] = (uint8_t)mine;
    if (mine <= it) return;
    const long long st[3] = {(long long)g.pz * g.ny, g.pz, 1};
    const int pos[3] = {x, y, z}, lim[3] = {g.nx, g.ny, g.nz};
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    int cnt = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
#pragma unroll
        for (int o = -1; o <= 1; o += 2) {
            const int q = pos[a] + o;
            if (q < 0 || q >= lim[a]) continue;
            const long long cn = c + o * st[a];
            if (vld(cn) > it) continue;
            s0 += v0[cn];
            s1 += v1[cn];
            s2 += v2[cn];
            cnt++;
        }
    }
    if (cnt > 0) {
        const float inv = (float)cnt;
        if (x + 1 < g.nx && flags[c + st[0]] != C_WATER) v0[c] = s0 / inv;
        if (y + 1 < g.ny && flags[c + st[1]] != C_WATER) v1[c] = s1 / inv;
        if (z + 1 < g.nz && flags[c + st[2]] != C_WATER) v2[c] = s2 / inv;
        valid[c] = (uint8_t)(it + 1);
    }
}

// ---- pressure application (applyPressureToVelocities,
//      bridsonSolverGrid.cpp:295-327) -------------------------------------------
// Each cell updates its own three faces: a fluid cell with a non-SOLID +a
// neighbour adds scale*(p_c - p_n) (p_n = 0 for AIR); an AIR cell with a fluid
// +a neighbour subtracts scale*p_n.
// BasicMacGrid::solveIncompressibilityParallel (basicMacGrid.cpp:16-88): one
// colour of the red-black SOR.  A WATER cell with s non-solid neighbours
// spreads d = 1.98 (-div v2 [+ density term]) / s over its six faces (a face
// towards a SOLID neighbour stays).  Cells of one colour share no face, so the
// update is order-free and deterministic.  parity: (x + y + z) & 1 of the
// colour (the reference runs odd, then even).
__global__ void k_sor(GridGeom g, const uint8_t* flags, float* vx, float* vy, float* vz, const float* avg,
                      int pressure_enabled, float avg_pressure, float pressure_k, int parity, float omega) {
    const int ix = (g.nx - 2), iy = (g.ny - 2), izh = (g.nz - 1) / 2;  // z pairs per interior row
    const long long total = (long long)ix * iy * izh;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int x = 1 + (int)(t / ((long long)iy * izh));
    const int y = 1 + (int)((t / izh) % iy);
    const int z = 1 + ((x + y + 1 + parity) & 1) + 2 * (int)(t % izh);
    if (z >= g.nz - 1) return;
    const long long c = gidx(g, x, y, z);
    if (flags[c] != C_WATER) return;
    const long long sx = (long long)g.pz * g.ny, sy = g.pz;
    const int s1 = flags[c + 1] != C_SOLID, s2 = flags[c - 1] != C_SOLID;
    const int s3 = flags[c + sy] != C_SOLID, s4 = flags[c - sy] != C_SOLID;
    const int s5 = flags[c + sx] != C_SOLID, s6 = flags[c - sx] != C_SOLID;
    const int s = s1 + s2 + s3 + s4 + s5 + s6;
    if (s == 0) return;
    float d = -vx[c] - vy[c] - vz[c] + vx[c - sx] + vy[c - sy] + vz[c - 1];
    if (pressure_enabled) d += (avg[c] - avg_pressure) * pressure_k;
    d = d * omega / (float)s;
    if (s1) vz[c] += d;
    if (s2) vz[c - 1] -= d;
    if (s3) vy[c] += d;
    if (s4) vy[c - sy] -= d;
    if (s5) vx[c] += d;
    if (s6) vx[c - sx] -= d;
}

__global__ void k_apply_pressure(GridGeom g, const uint8_t* flags, const double* p, double scale,
                                 float* v0, float* v1, float* v2) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    if (z >= g.nz) return;
    const uint8_t fc = flags[c];
    if (fc == C_SOLID) return;
    const long long st[3] = {(long long)g.pz * g.ny, g.pz, 1};
    const int pos[3] = {x, y, z}, lim[3] = {g.nx, g.ny, g.nz};
    float* vv[3] = {v0, v1, v2};
    const double pc = (fc == C_WATER) ? p[c] : 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (pos[a] + 1 >= lim[a]) continue;
        const long long cn = c + st[a];
        const uint8_t fn = flags[cn];
        if (fc == C_WATER) {
            if (fn == C_SOLID) continue;
            const double pn = (fn == C_WATER) ? p[cn] : 0.0;
            vv[a][c] = (float)((double)vv[a][c] + scale * (pc - pn));
        } else if (fn == C_WATER) {  // fc == AIR
            vv[a][c] = (float)((double)vv[a][c] - scale * p[cn]);
        }
    }
}

// ---- layout conversions ------------------------------------------------------
template <typename T>
__global__ void k_pad_to_dense(GridGeom g, const T* src, T* dst) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)g.nx * g.ny * g.nz;
    if (j >= n) return;
    const int z = (int)(j % g.nz);
    const long long row = j / g.nz;
    dst[j] = src[row * g.pz + z];
}
template <typename T>
__global__ void k_dense_to_pad(GridGeom g, const T* src, T* dst) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)g.nx * g.ny * g.nz;
    if (j >= n) return;
    const int z = (int)(j % g.nz);
    const long long row = j / g.nz;
    dst[row * g.pz + z] = src[j];
}
__global__ void k_counts(GridGeom g, const int* cstart, int* out) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)g.nx * g.ny * g.nz;
    if (j >= n) return;
    const int z = (int)(j % g.nz);
    const long long c = (j / g.nz) * g.pz + z;
    out[j] = cstart[c + 1] - cstart[c];
}
__global__ void k_copy_phi(GridGeom g, const double* phi, float* out) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)g.nx * g.ny * g.nz;
    if (j >= n) return;
    const int z = (int)(j % g.nz);
    out[j] = (float)phi[(j / g.nz) * g.pz + z];
}

}  // namespace

int launch_obstacle(fsim_ctx* ctx, const fsim_obstacle& ob) {
    const GridGeom& g = ctx->g;
    ObsGeom o;
    const double hinv = g.hinvd, hinv_a[3] = {g.hinvd, g.hinvd, g.hzinvd};
    const double cx = ob.pos[0] * hinv, cy = ob.pos[1] * hinv, cz = ob.pos[2] * g.hzinvd;
    for (int a = 0; a < 3; a++) o.speed[a] = (float)ob.speed[a];
    const int nn[3] = {g.nx, g.ny, g.nz};
    const double cc[3] = {cx, cy, cz};
    if (ob.type == FSIM_OBS_SPHERE || ob.type == FSIM_OBS_SOURCE) {
        o.kind = 0;
        const double r = hinv * ob.r;  // cellDInv.x * r, on every axis
        o.cx = cx; o.cy = cy; o.cz = cz;
        o.r2 = r * r;
        for (int a = 0; a < 3; a++) {
            o.mn[a] = (int)std::max(cc[a] - r, 1.0);
            o.mx[a] = (int)std::min(cc[a] + r, nn[a] - 2.0);
        }
    } else if (ob.type == FSIM_OBS_BOX) {
        o.kind = 1;
        o.cx = o.cy = o.cz = o.r2 = 0;
        for (int a = 0; a < 3; a++) {
            const double d = ob.size[a] * hinv_a[a] * 0.5;
            o.mn[a] = (int)std::max(std::round(cc[a] - d), 1.0);
            o.mx[a] = (int)std::min(std::round(cc[a] + d), nn[a] - 1.0);
        }
    } else {
        return 0;  // sinks and disc sources are not rasterised (macGrid.cpp:235)
    }
    // extent of the index box (sphere bounds inclusive, box exclusive)
    int ext[3];
    for (int a = 0; a < 3; a++) {
        ext[a] = (o.kind == 0) ? o.mx[a] - o.mn[a] + 1 : o.mx[a] - o.mn[a];
        if (ext[a] <= 0) return 0;
    }
    const int ex = ext[0] + 1, ey = ext[1] + 1, ez = ext[2] + 1;
    k_obstacle_faces<<<ceil_div((long long)ex * ey * ez, 256), 256, 0, ctx->stream>>>(
        g, o, ctx->flags, ctx->u[0], ctx->u[1], ctx->u[2], ex, ey, ez);
    k_obstacle_cells<<<ceil_div((long long)ext[0] * ext[1] * ext[2], 256), 256, 0, ctx->stream>>>(
        g, o, ctx->flags, ext[0], ext[1], ext[2]);
    return 2;
}

namespace {
__global__ void k_fetch_small(unsigned* dst, const unsigned* src, int words) {
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    __threadfence_system();
}
}  // namespace

void fetch_small(void* host, const void* dev, int bytes, cudaStream_t s) {
    // every caller's buffers are 4-byte aligned and a whole number of words
    k_fetch_small<<<1, 32, 0, s>>>(static_cast<unsigned*>(host), static_cast<const unsigned*>(dev), (bytes + 3) / 4);
}

void launch_prep(fsim_ctx* ctx, int walls, int post, float gravity_inc) {
    const GridGeom& g = ctx->g;
    ctx->launches += 1;
    k_prep<<<ceil_div(g.ncell, 256), 256, 0, ctx->stream>>>(
        g, ctx->prm.top_solid, walls, post, gravity_inc, ctx->flags, ctx->u[0], ctx->u[1], ctx->u[2],
        ctx->v2[0], ctx->v2[1], ctx->v2[2]);
}

void launch_extrapolate(fsim_ctx* ctx) {
    const GridGeom& g = ctx->g;
    ctx->launches += 2;
    for (int it = 0; it < 2; it++)
        k_extrapolate<<<ceil_div(g.ncell, 256), 256, 0, ctx->stream>>>(g, it, ctx->flags, ctx->valid,
                                                                       ctx->v2[0], ctx->v2[1], ctx->v2[2]);
}

int launch_sor(fsim_ctx* ctx, int iters) {
    const GridGeom& g = ctx->g;
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return 0;
    const long long total = (long long)(g.nx - 2) * (g.ny - 2) * ((g.nz - 1) / 2);
    const fsim_params& P = ctx->prm;
    for (int n = 0; n < iters; n++) {
        for (int parity = 1; parity >= 0; parity--)
            k_sor<<<ceil_div(total, 256), 256, 0, ctx->stream>>>(g, ctx->flags, ctx->v2[0], ctx->v2[1], ctx->v2[2],
                                                                  ctx->avg, P.pressure_enabled,
                                                                  (float)P.average_pressure, (float)P.pressure_k,
                                                                  parity, 1.98f);
    }
    ctx->launches += 2LL * iters;
    return iters;
}

void launch_apply_pressure(fsim_ctx* ctx, double dt) {
    const GridGeom& g = ctx->g;
    ctx->launches += 1;
    const double scale = dt / (ctx->prm.fluid_density * g.hd);
    k_apply_pressure<<<ceil_div(g.ncell, 256), 256, 0, ctx->stream>>>(g, ctx->flags, ctx->sv.phi, scale,
                                                                      ctx->v2[0], ctx->v2[1], ctx->v2[2]);
}

void launch_pad_to_dense(const GridGeom& g, const void* src, void* dst, int elem, cudaStream_t s) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const int nb = ceil_div(n, 256);
    if (elem == 1) k_pad_to_dense<uint8_t><<<nb, 256, 0, s>>>(g, (const uint8_t*)src, (uint8_t*)dst);
    else if (elem == 4) k_pad_to_dense<float><<<nb, 256, 0, s>>>(g, (const float*)src, (float*)dst);
    else k_pad_to_dense<double><<<nb, 256, 0, s>>>(g, (const double*)src, (double*)dst);
}

void launch_dense_to_pad(const GridGeom& g, const void* src, void* dst, int elem, cudaStream_t s) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const int nb = ceil_div(n, 256);
    if (elem == 1) k_dense_to_pad<uint8_t><<<nb, 256, 0, s>>>(g, (const uint8_t*)src, (uint8_t*)dst);
    else if (elem == 4) k_dense_to_pad<float><<<nb, 256, 0, s>>>(g, (const float*)src, (float*)dst);
    else k_dense_to_pad<double><<<nb, 256, 0, s>>>(g, (const double*)src, (double*)dst);
}

void launch_counts(const GridGeom& g, const int* cstart, int* out, cudaStream_t s) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_counts<<<ceil_div(n, 256), 256, 0, s>>>(g, cstart, out);
}

void launch_copy_phi(const GridGeom& g, const double* phi, float* out, cudaStream_t s) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_copy_phi<<<ceil_div(n, 256), 256, 0, s>>>(g, phi, out);
}
