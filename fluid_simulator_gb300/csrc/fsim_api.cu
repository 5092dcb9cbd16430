// fsim_api.cu -- the C ABI declared in include/fsim.h: context lifecycle,
// particle and grid exchange, and the per-step orchestration that replaces
// Simulator::simulate (simulator.cpp:51-100).
//
// Step order (all on the context's stream):
//   spawn -> advect + push-out + cell keys (one kernel) -> scan + scatter
//   (counting sort by cell) -> P2G + marking (tile kernel) -> obstacles ->
//   walls + v2/gravity (one kernel) -> pressure solve + apply -> extrapolation
//   (2 passes) -> G2P (tile kernel; writes the particles in sorted order into
//   the second buffer, which becomes current).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fsim_ctx.h"

namespace {

// ---- AoS <-> SoA ------------------------------------------------------------
__global__ void k_aos_to_soa(const float* pos, const float* vel, const float* c, long long n, ParticleBuf d,
                             long long first, uint32_t id0, int ids) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long j = first + i;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        d.p[a][j] = pos[3 * i + a];
        d.v[a][j] = vel ? vel[3 * i + a] : 0.f;
    }
#pragma unroll
    for (int a = 0; a < 9; a++) d.c[a][j] = c ? c[9 * i + a] : 0.f;
    if (ids) d.id[j] = id0 + (uint32_t)i;
}

__global__ void k_soa_to_aos(ParticleBuf s, long long n, const int* dst_index, float* pos, float* vel, float* c) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long j = dst_index ? dst_index[i] : i;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (pos) pos[3 * j + a] = s.p[a][i];
        if (vel) vel[3 * j + a] = s.v[a][i];
    }
    if (c)
#pragma unroll
        for (int a = 0; a < 9; a++) c[9 * j + a] = s.c[a][i];
}

__global__ void k_mark_ids(const uint32_t* id, long long n, int* present) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) present[id[i]] = 1;
}
__global__ void k_id_rank(const uint32_t* id, long long n, const int* prefix, int* out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = prefix[id[i]];
}
__global__ void k_fill_u8(uint8_t* p, long long n, uint8_t v) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
// initial cell types: padding SOLID, border SOLID (MacGrid ctor), rest AIR
__global__ void k_init_flags(GridGeom g, int top_solid, uint8_t* f) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    bool solid = z >= g.nz || x == 0 || x == g.nx - 1 || y == 0 || (top_solid && y == g.ny - 1) || z == 0 ||
                 z == g.nz - 1;
    f[c] = solid ? C_SOLID : C_AIR;
}
__global__ void k_dense_f32_to_f64_pad(GridGeom g, const float* src, double* dst) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)g.nx * g.ny * g.nz;
    if (j >= n) return;
    dst[(j / g.nz) * g.pz + (j % g.nz)] = (double)src[j];
}

int set_error(fsim_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

#define CHECK_LAUNCH(ctx)                                                                  \
    do {                                                                                   \
        cudaError_t e_ = cudaGetLastError();                                               \
        if (e_ != cudaSuccess) return set_error(ctx, FSIM_E_CUDA, cudaGetErrorString(e_)); \
    } while (0)

size_t buf_words(long long cap) { return (size_t)cap * 16; }

void bind_buf(ParticleBuf& b, void* mem, long long cap) {
    float* f = (float*)mem;
    for (int a = 0; a < 3; a++) b.p[a] = f + (size_t)a * cap;
    for (int a = 0; a < 3; a++) b.v[a] = f + (size_t)(3 + a) * cap;
    for (int a = 0; a < 9; a++) b.c[a] = f + (size_t)(6 + a) * cap;
    b.id = (uint32_t*)(f + (size_t)15 * cap);
}

int ensure_capacity(fsim_ctx* ctx, long long need) {
    if (need <= ctx->cap) return FSIM_OK;
    long long cap = std::max<long long>(need, std::max<long long>(2 * ctx->cap, 1024));
    void* nm[2] = {nullptr, nullptr};
    for (int k = 0; k < 2; k++) {
        if (cudaMalloc(&nm[k], buf_words(cap) * 4) != cudaSuccess) {
            cudaFree(nm[0]);
            cudaGetLastError();
            return set_error(ctx, FSIM_E_OOM, "particle buffer allocation failed");
        }
    }
    ParticleBuf nb[2];
    bind_buf(nb[0], nm[0], cap);
    bind_buf(nb[1], nm[1], cap);
    if (ctx->n > 0) {
        // copy the current buffer's 16 arrays
        const ParticleBuf& ob = ctx->buf[ctx->cur];
        const size_t bytes = (size_t)ctx->n * 4;
        for (int a = 0; a < 3; a++) {
            cudaMemcpyAsync(nb[0].p[a], ob.p[a], bytes, cudaMemcpyDeviceToDevice, ctx->stream);
            cudaMemcpyAsync(nb[0].v[a], ob.v[a], bytes, cudaMemcpyDeviceToDevice, ctx->stream);
        }
        for (int a = 0; a < 9; a++)
            cudaMemcpyAsync(nb[0].c[a], ob.c[a], bytes, cudaMemcpyDeviceToDevice, ctx->stream);
        cudaMemcpyAsync(nb[0].id, ob.id, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    }
    uint32_t *key = nullptr, *rank = nullptr, *perm = nullptr;
    if (cudaMalloc(&key, cap * 4) != cudaSuccess || cudaMalloc(&rank, cap * 4) != cudaSuccess ||
        cudaMalloc(&perm, cap * 4) != cudaSuccess) {
        cudaFree(nm[0]); cudaFree(nm[1]); cudaFree(key); cudaFree(rank); cudaFree(perm);
        cudaGetLastError();
        return set_error(ctx, FSIM_E_OOM, "particle index allocation failed");
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->buf_mem[0]);
    cudaFree(ctx->buf_mem[1]);
    cudaFree(ctx->key); cudaFree(ctx->rank); cudaFree(ctx->perm);
    ctx->buf_mem[0] = nm[0];
    ctx->buf_mem[1] = nm[1];
    ctx->buf[0] = nb[0];
    ctx->buf[1] = nb[1];
    ctx->cur = 0;
    ctx->key = key; ctx->rank = rank; ctx->perm = perm;
    ctx->cap = cap;
    ctx->sorted = false;
    return FSIM_OK;
}

DevObstacle to_dev(const fsim_ctx* ctx, const fsim_obstacle& o) {
    DevObstacle d{};
    d.type = o.type;
    for (int a = 0; a < 3; a++) {
        d.pos[a] = (float)o.pos[a];
        d.speed[a] = (float)o.speed[a];
        d.size[a] = (float)o.size[a];
    }
    d.r = (float)o.r;
    if (o.type == FSIM_OBS_BOX) {
        // MacGrid::getMinMaxRect (macGrid.h:139-145) widened by the particle radius
        const GridGeom& g = ctx->g;
        const int nn[3] = {g.nx, g.ny, g.nz};
        const double pr = ctx->prm.particle_r;
        const double hh[3] = {g.hd, g.hd, g.hzd}, hi[3] = {g.hinvd, g.hinvd, g.hzinvd};
        for (int a = 0; a < 3; a++) {
            const double c = o.pos[a] * hi[a], dd = o.size[a] * hi[a] * 0.5;
            const int mn = (int)std::max(std::round(c - dd), 1.0);
            const int mx = (int)std::min(std::round(c + dd), nn[a] - 1.0);
            d.box_lo[a] = (float)((double)mn * hh[a] - pr);
            d.box_hi[a] = (float)((double)mx * hh[a] + pr);
        }
    }
    return d;
}

void fill_advect_args(fsim_ctx* ctx, AdvectArgs& a, double dt) {
    std::memset(&a, 0, sizeof(a));
    a.p = ctx->buf[ctx->cur];
    a.n = ctx->n;
    a.dt = (float)dt;
    const GridGeom& g = ctx->g;
    const double pr = ctx->prm.particle_r;
    for (int k = 0; k < 3; k++) {
        const double hk = k == 2 ? g.hzd : g.hd;
        // gridLow (simulator.cpp:140): no radius margin on z in 2D mode
        const double lo = hk + (k == 2 && g.two_d ? 0.0 : pr) * 1.01;
        const double plo = hk + pr * 1.01;  // particleLow (simulator.cpp:257)
        a.lo[k] = (float)lo;
        a.hi[k] = (float)(g.dims[k] - lo);
        a.plo[k] = (float)plo;
        a.phi[k] = (float)(g.dims[k] - plo);
    }
    a.pr = (float)pr;
    a.despawn = ctx->prm.despawning_enabled;
    int n = 0;
    for (const auto& o : ctx->obs) {
        if (o.type == FSIM_OBS_DISC_SOURCE) continue;
        if (n < FSIM_MAX_OBS) a.obs[n++] = to_dev(ctx, o);
    }
    a.nobs = n;
    a.g = g;
    a.key = ctx->key;
    a.rank = ctx->rank;
    a.count = ctx->count;
}

// counting sort by cell of the current buffer (keys from do_key)
int sort_by_cell(fsim_ctx* ctx) {
    launch_scan(ctx->count, ctx->cstart, ctx->g.ncell, ctx->scan_blocks, ctx->stream);
    launch_scatter(ctx->key, ctx->rank, ctx->cstart, ctx->perm, ctx->n, ctx->g.ncell, ctx->stream);
    ctx->launches += 3 + (ctx->n > 0 ? 2 : 0);
    fetch_small(ctx->h_misc, ctx->cstart + ctx->g.ncell, sizeof(int), ctx->stream);
    ctx->launches += 1;
    CHECK_LAUNCH(ctx);
    ctx->sorted = true;
    return FSIM_OK;
}

int run_keys(fsim_ctx* ctx, int do_advect, int do_push, int do_stop, double dt) {
    AdvectArgs a;
    fill_advect_args(ctx, a, dt);
    a.do_advect = do_advect;
    a.do_push = do_push;
    a.do_stop = do_stop;
    a.do_key = 1;
    FSIM_CUDA_TRY(ctx, cudaMemsetAsync(ctx->count, 0, (size_t)ctx->g.ncell * sizeof(int), ctx->stream));
    launch_advect(a, ctx->stream);
    ctx->launches += ctx->n > 0 ? 1 : 0;
    CHECK_LAUNCH(ctx);
    return sort_by_cell(ctx);
}

// HashedParticles::pushParticlesApart (hashedParticles.cpp:64-107), Jacobi
// semantics (k_push_apart); needs the cell sort of the current positions
int push_apart_pass(fsim_ctx* ctx) {
    const GridGeom& g = ctx->g;
    const double pr = ctx->prm.particle_r;
    if (2.0 * pr > std::min(g.hd, g.hzd))
        return set_error(ctx, FSIM_E_UNSUPPORTED, "push-apart needs particle_r <= h/2 (neighbours within one cell)");
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        const double low = (k == 2 ? g.hzd : g.hd) + pr * 1.01;  // particleLow (hashedParticles.cpp:67)
        lo[k] = (float)low;
        hi[k] = (float)(g.dims[k] - low);
    }
    float* tmp[3] = {ctx->buf[1 - ctx->cur].p[0], ctx->buf[1 - ctx->cur].p[1], ctx->buf[1 - ctx->cur].p[2]};
    launch_push_apart(ctx->buf[ctx->cur], ctx->perm, ctx->cstart, g, ctx->n, pr, lo, hi, tmp, ctx->stream);
    ctx->launches += ctx->n > 0 ? 1 : 0;
    CHECK_LAUNCH(ctx);
    for (int k = 0; k < 3; k++)
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->buf[ctx->cur].p[k], tmp[k], (size_t)ctx->n * sizeof(float),
                                           cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->sorted = false;
    return FSIM_OK;
}

int run_particle_only(fsim_ctx* ctx, int do_advect, int do_push, int do_stop, double dt) {
    AdvectArgs a;
    fill_advect_args(ctx, a, dt);
    a.do_advect = do_advect;
    a.do_push = do_push;
    a.do_stop = do_stop;
    a.do_key = 0;
    launch_advect(a, ctx->stream);
    ctx->launches += ctx->n > 0 ? 1 : 0;
    CHECK_LAUNCH(ctx);
    ctx->sorted = false;
    return FSIM_OK;
}

// host count of live particles after the last sort (h_misc holds cstart[ncell])
int finish_sort_count(fsim_ctx* ctx) {
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return FSIM_OK;
}

int do_spawn(fsim_ctx* ctx, double dt) {
    // count on the host (Simulator::spawnParticles, simulator.cpp:106-125)
    struct Job {
        int obs;
        int count;
        std::vector<int> cells;
        int cy;
    };
    std::vector<Job> jobs;
    long long total = 0;
    const GridGeom& g = ctx->g;
    for (size_t k = 0; k < ctx->obs.size(); k++) {
        fsim_obstacle& o = ctx->obs[k];
        if (o.type == FSIM_OBS_SOURCE) {
            const double nd = o.spawn_rate * dt + o.last_spawn_fraction;
            const int num = (int)nd;
            o.last_spawn_fraction = nd - num;
            if (num > 0) {
                jobs.push_back({(int)k, num, {}, 0});
                total += num;
            }
        } else if (o.type == FSIM_OBS_DISC_SOURCE) {
            Job j{(int)k, 0, {}, (int)(o.pos[1] * g.hinvd)};
            const double cx = o.pos[0] * g.hinvd, cz = o.pos[2] * g.hzinvd, r = o.r * g.hinvd;
            for (int x = 1; x < g.nx - 1; x++)
                for (int z = 1; z < g.nz - 1; z++) {
                    const double dx = x + 0.5 - cx, dz = z + 0.5 - cz;
                    if (dx * dx + dz * dz <= r * r) {
                        j.cells.push_back(x);
                        j.cells.push_back(z);
                    }
                }
            j.count = (int)(j.cells.size() / 2) * 8;
            if (j.count > 0 && j.cy >= 1 && j.cy < g.ny - 1) {
                total += j.count;
                jobs.push_back(std::move(j));
            }
        }
    }
    if (total == 0) return FSIM_OK;
    int rc = ensure_capacity(ctx, ctx->n + total);
    if (rc) return rc;
    // the step's disc cell lists go to mapped pinned memory (grown rarely); the
    // previous step's spawn kernels finished before that step returned
    long long list_ints = 0;
    for (const auto& j : jobs) list_ints += (long long)j.cells.size();
    if (list_ints > ctx->disc_cells_cap) {
        if (ctx->disc_cells_host) cudaFreeHost(ctx->disc_cells_host);
        ctx->disc_cells_host = nullptr;
        ctx->disc_cells_dev = nullptr;
        ctx->disc_cells_cap = 0;
        const long long cap = std::max<long long>(2 * list_ints, 1024);
        FSIM_CUDA_TRY(ctx, cudaHostAlloc((void**)&ctx->disc_cells_host, (size_t)cap * sizeof(int),
                                         cudaHostAllocMapped));
        FSIM_CUDA_TRY(ctx, cudaHostGetDevicePointer((void**)&ctx->disc_cells_dev, ctx->disc_cells_host, 0));
        ctx->disc_cells_cap = cap;
    }
    long long list_off = 0;
    const bool ids = ctx->prm.track_ids != 0;
    for (auto& j : jobs) {
        const fsim_obstacle& o = ctx->obs[j.obs];
        const uint64_t seed = 0x5eedull + ctx->spawn_counter++;
        if (o.type == FSIM_OBS_SOURCE) {
            launch_spawn_sphere(ctx->buf[ctx->cur], ctx->n, j.count, o, ctx->prm.particle_r, seed, ctx->next_id,
                                ids, ctx->stream);
            ctx->launches += 1;
        } else {
            std::memcpy(ctx->disc_cells_host + list_off, j.cells.data(), j.cells.size() * sizeof(int));
            launch_spawn_disc(ctx->buf[ctx->cur], ctx->n, (int)(j.cells.size() / 2), o, g, j.cy,
                              ctx->disc_cells_dev + list_off, seed, ctx->next_id, ids, ctx->stream);
            list_off += (long long)j.cells.size();
            ctx->launches += 1;
        }
        ctx->n += j.count;
        ctx->next_id += (uint32_t)j.count;
    }
    CHECK_LAUNCH(ctx);
    ctx->sorted = false;
    return FSIM_OK;
}

int check_device_error(fsim_ctx* ctx) {
    unsigned* he = reinterpret_cast<unsigned*>(&ctx->h_misc[2]);
    fetch_small(he, ctx->d_err, sizeof(unsigned), ctx->stream);
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const unsigned e = *he;
    if (e & FSIM_DERR_TMA_TIMEOUT) {
        cudaMemset(ctx->d_err, 0, sizeof(unsigned));
        return set_error(ctx, FSIM_E_TIMEOUT, "G2P tile load wait timed out");
    }
    return FSIM_OK;
}

// stage time between two recorded events; a pair that was not recorded reads 0
// (and its error is cleared, so a timing query never fails a step)
float elapsed(fsim_ctx* ctx, int a, int b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.f;
    }
    return ms;
}

int validate_params(const fsim_params* p, std::string& why) {
    if (p->transfer < FSIM_PIC || p->transfer > FSIM_APIC) { why = "transfer type"; return FSIM_E_INVALID; }
    if (p->max_iters < 0) { why = "max_iters"; return FSIM_E_INVALID; }
    if (!(p->fluid_density > 0)) { why = "fluid_density"; return FSIM_E_INVALID; }
    if (p->precision < FSIM_PREC_MIXED || p->precision > FSIM_PREC_FP64) { why = "precision"; return FSIM_E_INVALID; }
    if (p->tol_mode != FSIM_TOL_ABS_MAX && p->tol_mode != FSIM_TOL_REL_L2) { why = "tol_mode"; return FSIM_E_INVALID; }
    if (p->warm_start < FSIM_WARM_ZERO || p->warm_start > FSIM_WARM_LEARNED_RESIDUAL) {
        why = "warm_start";
        return FSIM_E_INVALID;
    }
    if (p->mg_boundary_sweeps < -1 || p->mg_boundary_sweeps > 8) { why = "mg_boundary_sweeps"; return FSIM_E_INVALID; }
    return FSIM_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

int fsim_create(const fsim_grid_desc* gd, const fsim_params* params, fsim_ctx** out) {
    if (!gd || !params || !out) return FSIM_E_INVALID;
    *out = nullptr;
    if (!(gd->resolution > 0) || !(gd->dims[0] > 0) || !(gd->dims[1] > 0) || !(gd->dims[2] > 0))
        return FSIM_E_INVALID;
    std::string why;
    int rc = validate_params(params, why);
    if (rc) return rc;
    fsim_ctx* ctx = new (std::nothrow) fsim_ctx();
    if (!ctx) return FSIM_E_OOM;
    ctx->prm = *params;
    // MacGrid ctor (macGrid.cpp:9-13): cellD = 1 / resolution (resolution passed
    // as float); in 2D mode the z axis is 3 cells of targetDimensions.z / 3 and
    // keeps targetDimensions.z as its extent
    const double res = (double)(float)gd->resolution;
    GridGeom& g = ctx->g;
    g.hd = 1 / res;
    g.hinvd = 1.0 / g.hd;
    g.h = (float)g.hd;
    g.hinv = (float)g.hinvd;
    g.two_d = gd->two_d ? 1 : 0;
    g.hzd = g.two_d ? gd->dims[2] / 3 : g.hd;
    g.hzinvd = 1.0 / g.hzd;
    g.hz = (float)g.hzd;
    g.hzinv = (float)g.hzinvd;
    // the padded grid stays below 2^31 cells (32-bit cell coordinates in the
    // kernels; far above what the particle state of such a grid would need)
    const double cells = std::floor(gd->dims[0] / g.hd) * std::floor(gd->dims[1] / g.hd) *
                         (g.two_d ? 4.0 : std::floor(gd->dims[2] / g.hd) + 3.0);
    if (!(cells < 2147483648.0)) {
        delete ctx;
        return FSIM_E_INVALID;
    }
    g.nx = (int)(gd->dims[0] / g.hd);
    g.ny = (int)(gd->dims[1] / g.hd);
    g.nz = g.two_d ? 3 : (int)(gd->dims[2] / g.hd);
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) {
        delete ctx;
        return FSIM_E_INVALID;
    }
    g.pz = (g.nz + 3) & ~3;
    g.ncell = (long long)g.nx * g.ny * g.pz;
    g.dims[0] = g.nx * g.hd;
    g.dims[1] = g.ny * g.hd;
    g.dims[2] = g.two_d ? gd->dims[2] : g.nz * g.hd;
    g.zc = (float)(gd->dims[2] / 2);
    if (!(ctx->prm.particle_r > 0)) ctx->prm.particle_r = g.hd / 4.0;

    auto fail = [&](int code, const char* msg) {
        fsim_destroy(ctx);
        (void)msg;
        return code;
    };
    if (cudaGetDevice(&ctx->device) != cudaSuccess) return fail(FSIM_E_CUDA, "no device");
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(FSIM_E_CUDA, "stream");
    const size_t nc = (size_t)g.ncell;
    bool ok = cudaMalloc(&ctx->flags, nc) == cudaSuccess && cudaMalloc(&ctx->valid, nc) == cudaSuccess &&
              cudaMalloc(&ctx->avg, nc * 4) == cudaSuccess && cudaMalloc(&ctx->count, nc * 4) == cudaSuccess &&
              cudaMalloc(&ctx->cstart, (nc + 1) * 4) == cudaSuccess &&
              cudaMalloc(&ctx->scan_blocks, ((nc + 4095) / 4096 + 1) * 4) == cudaSuccess &&
              cudaMalloc(&ctx->d_err, sizeof(unsigned)) == cudaSuccess &&
              cudaMalloc(&ctx->d_misc, 64) == cudaSuccess && cudaMallocHost(&ctx->h_misc, 64) == cudaSuccess;
    for (int a = 0; a < 3 && ok; a++)
        ok = cudaMalloc(&ctx->u[a], nc * 4) == cudaSuccess && cudaMalloc(&ctx->v2[a], nc * 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return fail(FSIM_E_OOM, "grid allocation");
    }
    for (int a = 0; a < 3; a++) {
        cudaMemset(ctx->u[a], 0, nc * 4);
        cudaMemset(ctx->v2[a], 0, nc * 4);
    }
    cudaMemset(ctx->avg, 0, nc * 4);
    cudaMemset(ctx->count, 0, nc * 4);
    cudaMemset(ctx->cstart, 0, (nc + 1) * 4);
    cudaMemset(ctx->d_err, 0, sizeof(unsigned));
    cudaMemset(ctx->d_misc, 0, 64);  // [0..1]: P2G work counters (each launch leaves them at zero)
    k_init_flags<<<ceil_div(g.ncell, 256), 256, 0, ctx->stream>>>(g, ctx->prm.top_solid, ctx->flags);
    if (solver_alloc(ctx) != FSIM_OK) return fail(FSIM_E_OOM, "solver allocation");
    if (!make_tensor_maps(ctx)) return fail(FSIM_E_CUDA, "tensor maps");
    for (int k = 0; k < EV_COUNT; k++) cudaEventCreate(&ctx->ev[k]);
    ctx->events = true;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(FSIM_E_CUDA, "init");
    *out = ctx;
    return FSIM_OK;
}

int fsim_destroy(fsim_ctx* ctx) {
    if (!ctx) return FSIM_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        for (int k = 0; k < 2; k++) {
            cudaFree(ctx->gfx_stage[k]);
            if (ctx->gfx_ready[k]) cudaEventDestroy(ctx->gfx_ready[k]);
            if (ctx->gfx_done[k]) cudaEventDestroy(ctx->gfx_done[k]);
        }
        cudaStreamDestroy(ctx->copy_stream);
    }
    cudaFree(ctx->buf_mem[0]);
    cudaFree(ctx->buf_mem[1]);
    cudaFree(ctx->key); cudaFree(ctx->rank); cudaFree(ctx->perm);
    cudaFree(ctx->count); cudaFree(ctx->cstart); cudaFree(ctx->scan_blocks);
    cudaFree(ctx->flags); cudaFree(ctx->valid); cudaFree(ctx->avg);
    for (int a = 0; a < 3; a++) { cudaFree(ctx->u[a]); cudaFree(ctx->v2[a]); }
    cudaFree(ctx->d_err); cudaFree(ctx->d_misc); cudaFreeHost(ctx->h_misc);
    if (ctx->disc_cells_host) cudaFreeHost(ctx->disc_cells_host);
    solver_free(ctx);
    if (ctx->events)
        for (int k = 0; k < EV_COUNT; k++) cudaEventDestroy(ctx->ev[k]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FSIM_OK;
}

int fsim_set_params(fsim_ctx* ctx, const fsim_params* p) {
    if (!ctx || !p) return FSIM_E_INVALID;
    std::string why;
    int rc = validate_params(p, why);
    if (rc) return set_error(ctx, rc, why);
    const bool ids_before = ctx->prm.track_ids != 0;
    ctx->prm = *p;
    if (!(ctx->prm.particle_r > 0)) ctx->prm.particle_r = ctx->g.hd / 4.0;
    if (ctx->prm.track_ids && !ids_before) {
        // ids start counting from the current order
        return set_error(ctx, FSIM_E_STATE, "track_ids must be set at creation");
    }
    return FSIM_OK;
}

int fsim_get_params(fsim_ctx* ctx, fsim_params* out) {
    if (!ctx || !out) return FSIM_E_INVALID;
    *out = ctx->prm;
    return FSIM_OK;
}

int fsim_grid_info(fsim_ctx* ctx, int* n3, double* h3, double* dims3) {
    if (!ctx) return FSIM_E_INVALID;
    if (n3) { n3[0] = ctx->g.nx; n3[1] = ctx->g.ny; n3[2] = ctx->g.nz; }
    if (h3) { h3[0] = h3[1] = ctx->g.hd; h3[2] = ctx->g.hzd; }
    if (dims3) for (int a = 0; a < 3; a++) dims3[a] = ctx->g.dims[a];
    return FSIM_OK;
}

const char* fsim_last_error(fsim_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* fsim_stream(fsim_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int fsim_synchronize(fsim_ctx* ctx) {
    if (!ctx) return FSIM_E_INVALID;
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return FSIM_OK;
}

static int upload_particles(fsim_ctx* ctx, const float* pos, const float* vel, const float* c, int64_t n,
                            int where, long long first) {
    if (n <= 0) return FSIM_OK;
    const float *dp = pos, *dv = vel, *dc = c;
    void* tmp = nullptr;
    if (where == FSIM_HOST) {
        const size_t bytes = (size_t)n * 15 * 4;
        FSIM_CUDA_TRY(ctx, cudaMallocAsync(&tmp, bytes, ctx->stream));
        float* t = (float*)tmp;
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(t, pos, (size_t)n * 12, cudaMemcpyHostToDevice, ctx->stream));
        dp = t;
        dv = nullptr;
        dc = nullptr;
        if (vel) {
            FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(t + 3 * n, vel, (size_t)n * 12, cudaMemcpyHostToDevice, ctx->stream));
            dv = t + 3 * n;
        }
        if (c) {
            FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(t + 6 * n, c, (size_t)n * 36, cudaMemcpyHostToDevice, ctx->stream));
            dc = t + 6 * n;
        }
    }
    k_aos_to_soa<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(dp, dv, dc, n, ctx->buf[ctx->cur], first,
                                                            ctx->next_id, ctx->prm.track_ids ? 1 : 0);
    CHECK_LAUNCH(ctx);
    if (tmp) FSIM_CUDA_TRY(ctx, cudaFreeAsync(tmp, ctx->stream));
    ctx->next_id += (uint32_t)n;
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return FSIM_OK;
}

int fsim_set_particles(fsim_ctx* ctx, const float* pos, const float* vel, const float* c, int64_t n, int where) {
    if (!ctx || (n > 0 && !pos) || n < 0 || n >= (1ll << 31)) return FSIM_E_INVALID;
    int rc = ensure_capacity(ctx, n);
    if (rc) return rc;
    ctx->n = 0;
    ctx->next_id = 0;
    rc = upload_particles(ctx, pos, vel, c, n, where, 0);
    if (rc) return rc;
    ctx->n = n;
    ctx->sorted = false;
    return FSIM_OK;
}

int fsim_add_particles(fsim_ctx* ctx, const float* pos, const float* vel, const float* c, int64_t n, int where) {
    if (!ctx || (n > 0 && !pos) || n < 0 || ctx->n + n >= (1ll << 31)) return FSIM_E_INVALID;
    int rc = ensure_capacity(ctx, ctx->n + n);
    if (rc) return rc;
    rc = upload_particles(ctx, pos, vel, c, n, where, ctx->n);
    if (rc) return rc;
    ctx->n += n;
    ctx->sorted = false;
    return FSIM_OK;
}

int fsim_num_particles(fsim_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return FSIM_E_INVALID;
    *n = ctx->n;
    return FSIM_OK;
}

int fsim_get_particles(fsim_ctx* ctx, float* pos, float* vel, float* c, int64_t cap, int64_t* n_out, int where) {
    if (!ctx) return FSIM_E_INVALID;
    const long long n = ctx->n;
    if (n_out) *n_out = n;
    if (n == 0 || (!pos && !vel && !c)) return FSIM_OK;
    if (cap < n) return set_error(ctx, FSIM_E_INVALID, "output capacity below particle count");
    cudaStream_t s = ctx->stream;
    int* dst_index = nullptr;
    int* present = nullptr;
    if (ctx->prm.track_ids) {
        const long long m = (long long)ctx->next_id;
        FSIM_CUDA_TRY(ctx, cudaMallocAsync(&present, (size_t)(2 * m + 1 + n) * 4 + ((m + 4095) / 4096 + 1) * 4, s));
        int* prefix = present + m;
        dst_index = prefix + m + 1;
        int* blocks = dst_index + n;
        FSIM_CUDA_TRY(ctx, cudaMemsetAsync(present, 0, (size_t)m * 4, s));
        k_mark_ids<<<ceil_div(n, 256), 256, 0, s>>>(ctx->buf[ctx->cur].id, n, present);
        launch_scan(present, prefix, m, blocks, s);
        k_id_rank<<<ceil_div(n, 256), 256, 0, s>>>(ctx->buf[ctx->cur].id, n, prefix, dst_index);
        CHECK_LAUNCH(ctx);
    }
    float *dp = pos, *dv = vel, *dc = c;
    void* tmp = nullptr;
    if (where == FSIM_HOST) {
        FSIM_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * 15 * 4, s));
        float* t = (float*)tmp;
        dp = pos ? t : nullptr;
        dv = vel ? t + 3 * n : nullptr;
        dc = c ? t + 6 * n : nullptr;
    }
    k_soa_to_aos<<<ceil_div(n, 256), 256, 0, s>>>(ctx->buf[ctx->cur], n, dst_index, dp, dv, dc);
    CHECK_LAUNCH(ctx);
    if (where == FSIM_HOST) {
        if (pos) FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(pos, dp, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
        if (vel) FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(vel, dv, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
        if (c) FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(c, dc, (size_t)n * 36, cudaMemcpyDeviceToHost, s));
        FSIM_CUDA_TRY(ctx, cudaFreeAsync(tmp, s));
    }
    if (present) FSIM_CUDA_TRY(ctx, cudaFreeAsync(present, s));
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return FSIM_OK;
}

int fsim_set_obstacles(fsim_ctx* ctx, const fsim_obstacle* obs, int n) {
    if (!ctx || n < 0 || (n > 0 && !obs)) return FSIM_E_INVALID;
    int nonsrc = 0;
    for (int k = 0; k < n; k++) {
        if (obs[k].type < FSIM_OBS_SPHERE || obs[k].type > FSIM_OBS_BOX_SINK)
            return set_error(ctx, FSIM_E_INVALID, "obstacle type");
        if (obs[k].type != FSIM_OBS_DISC_SOURCE) nonsrc++;
    }
    if (nonsrc > FSIM_MAX_OBS) return set_error(ctx, FSIM_E_INVALID, "too many obstacles (max 32)");
    ctx->obs.assign(obs, obs + n);
    return FSIM_OK;
}

int fsim_get_obstacles(fsim_ctx* ctx, fsim_obstacle* obs, int cap, int* n) {
    if (!ctx) return FSIM_E_INVALID;
    if (n) *n = (int)ctx->obs.size();
    for (int k = 0; k < (int)ctx->obs.size() && k < cap; k++) obs[k] = ctx->obs[k];
    return FSIM_OK;
}

int fsim_stage(fsim_ctx* ctx, int stage, double dt, fsim_step_stats* stats) {
    if (!ctx) return FSIM_E_INVALID;
    int rc = FSIM_OK;
    const fsim_params& P = ctx->prm;
    switch (stage) {
        case FSIM_STAGE_SPAWN: rc = do_spawn(ctx, dt); break;
        case FSIM_STAGE_ADVECT:
            // advect, then compact deleted particles (order becomes cell order)
            if ((rc = run_keys(ctx, 1, 0, 0, dt))) return rc;
            launch_gather(ctx->buf[ctx->cur], ctx->buf[1 - ctx->cur], ctx->perm, ctx->cstart, ctx->g.ncell, ctx->n,
                          P.track_ids != 0, ctx->stream);
            CHECK_LAUNCH(ctx);
            FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            ctx->cur = 1 - ctx->cur;
            ctx->n = ctx->h_misc[0];
            ctx->sorted = false;
            break;
        case FSIM_STAGE_PUSH_APART:
            // sort the current positions (no movement), then one push-apart pass
            if ((rc = run_keys(ctx, 0, 0, 0, dt))) return rc;
            rc = push_apart_pass(ctx);
            break;
        case FSIM_STAGE_PUSH_OUT: rc = run_particle_only(ctx, 0, 1, 0, dt); break;
        case FSIM_STAGE_STOP: rc = run_particle_only(ctx, 0, 0, 1, dt); break;
        case FSIM_STAGE_P2G:
            if ((rc = run_keys(ctx, 0, 0, 0, dt))) return rc;
            launch_p2g(ctx);
            CHECK_LAUNCH(ctx);
            break;
        case FSIM_STAGE_MARK: break;
        case FSIM_STAGE_OBSTACLES:
            for (const auto& o : ctx->obs) ctx->launches += launch_obstacle(ctx, o);
            CHECK_LAUNCH(ctx);
            break;
        case FSIM_STAGE_WALLS: launch_prep(ctx, 1, 0, 0.f); CHECK_LAUNCH(ctx); break;
        case FSIM_STAGE_POST_P2G:
            launch_prep(ctx, 0, 1, P.gravity_enabled ? (float)((double)P.gravity * dt) : 0.f);
            CHECK_LAUNCH(ctx);
            break;
        case FSIM_STAGE_SOLVE: {
            fsim_step_stats tmp{};
            fsim_step_stats* sp = stats ? stats : &tmp;
            if (P.grid_solver == FSIM_SOLVER_SOR) {
                sp->pcg_iterations = launch_sor(ctx, P.max_iters);
                CHECK_LAUNCH(ctx);
                break;
            }
            const long long l0 = ctx->launches;
            rc = solve_pressure(ctx, dt, P.precision, P.tol_mode, P.residual_tol, P.max_iters, P.warm_start, sp,
                                nullptr, 1);
            sp->kernel_launches = (int)(ctx->launches - l0);
            break;
        }
        case FSIM_STAGE_EXTRAPOLATE: launch_extrapolate(ctx); CHECK_LAUNCH(ctx); break;
        case FSIM_STAGE_G2P:
            if (!ctx->sorted) return set_error(ctx, FSIM_E_STATE, "G2P needs the cell sort of a P2G stage");
            launch_g2p(ctx);
            CHECK_LAUNCH(ctx);
            FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            ctx->cur = 1 - ctx->cur;
            ctx->n = ctx->h_misc[0];
            ctx->sorted = false;
            if ((rc = check_device_error(ctx))) return rc;
            break;
        default: return set_error(ctx, FSIM_E_INVALID, "stage id");
    }
    if (rc) return rc;
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return FSIM_OK;
}

int fsim_step(fsim_ctx* ctx, double dt, fsim_step_stats* stats) {
    if (!ctx) return FSIM_E_INVALID;
    if (!(dt > 0)) return set_error(ctx, FSIM_E_INVALID, "dt must be positive");
    const fsim_params& P = ctx->prm;
    fsim_step_stats st{};
    const long long launches0 = ctx->launches;
    int rc;
    fsim_record(ctx, EV_START);
    if (P.spawning_enabled && (rc = do_spawn(ctx, dt))) return rc;
    // advect + push-out + stop + keys, then the counting sort
    if (P.push_apart_enabled) {
        // advect (+ sinks) with keys and a sort, push apart, then push-out /
        // stop with keys (deleted particles stay deleted) and the step's sort
        AdvectArgs a;
        fill_advect_args(ctx, a, dt);
        a.do_advect = 1;
        a.do_key = 1;
        FSIM_CUDA_TRY(ctx, cudaMemsetAsync(ctx->count, 0, (size_t)ctx->g.ncell * sizeof(int), ctx->stream));
        launch_advect(a, ctx->stream);
        ctx->launches += ctx->n > 0 ? 1 : 0;
        CHECK_LAUNCH(ctx);
        fsim_record(ctx, EV_ADVECT);
        if ((rc = sort_by_cell(ctx))) return rc;
        if ((rc = push_apart_pass(ctx))) return rc;
        fsim_record(ctx, EV_APART);
        fill_advect_args(ctx, a, dt);
        a.do_push = 1;
        a.do_stop = P.stop_particles;
        a.do_key = 1;
        a.keep_dead = 1;
        FSIM_CUDA_TRY(ctx, cudaMemsetAsync(ctx->count, 0, (size_t)ctx->g.ncell * sizeof(int), ctx->stream));
        launch_advect(a, ctx->stream);
        ctx->launches += ctx->n > 0 ? 1 : 0;
        CHECK_LAUNCH(ctx);
    } else {
        AdvectArgs a;
        fill_advect_args(ctx, a, dt);
        a.do_advect = 1;
        a.do_push = 1;
        a.do_stop = P.stop_particles;
        a.do_key = 1;
        FSIM_CUDA_TRY(ctx, cudaMemsetAsync(ctx->count, 0, (size_t)ctx->g.ncell * sizeof(int), ctx->stream));
        launch_advect(a, ctx->stream);
        ctx->launches += ctx->n > 0 ? 1 : 0;
        CHECK_LAUNCH(ctx);
        fsim_record(ctx, EV_ADVECT);
    }
    if ((rc = sort_by_cell(ctx))) return rc;
    fsim_record(ctx, EV_SORT);
    launch_p2g(ctx);
    CHECK_LAUNCH(ctx);
    fsim_record(ctx, EV_P2G);
    for (const auto& o : ctx->obs) ctx->launches += launch_obstacle(ctx, o);
    launch_prep(ctx, 1, 1, P.gravity_enabled ? (float)((double)P.gravity * dt) : 0.f);
    CHECK_LAUNCH(ctx);
    fsim_record(ctx, EV_PREP);
    if (P.grid_solver == FSIM_SOLVER_SOR) {
        fsim_record(ctx, EV_PCG_SETUP);  // no setup: keeps the stage timings defined
        st.pcg_iterations = launch_sor(ctx, P.max_iters);  // BasicMacGrid returns its iteration count
        CHECK_LAUNCH(ctx);
    } else {
        rc = solve_pressure(ctx, dt, P.precision, P.tol_mode, P.residual_tol, P.max_iters, P.warm_start, &st,
                            nullptr, 1);
        if (rc) return rc;
    }
    fsim_record(ctx, EV_SOLVE);
    launch_extrapolate(ctx);
    CHECK_LAUNCH(ctx);
    fsim_record(ctx, EV_EXTRAP);
    launch_g2p(ctx);
    CHECK_LAUNCH(ctx);
    fsim_record(ctx, EV_G2P);
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->cur = 1 - ctx->cur;
    ctx->n = ctx->h_misc[0];
    ctx->sorted = false;
    if ((rc = check_device_error(ctx))) return rc;
    if (stats) {
        st.num_particles = (int)ctx->n;
        st.kernel_launches = (int)(ctx->launches - launches0);
        if (P.timing) {
            st.ms_simulate_particles = elapsed(ctx, EV_START, EV_ADVECT);
            st.ms_push_apart = P.push_apart_enabled ? elapsed(ctx, EV_ADVECT, EV_APART) : 0.f;
            st.ms_p2g = elapsed(ctx, P.push_apart_enabled ? EV_APART : EV_ADVECT, EV_P2G);
            st.ms_p2g_kernel = elapsed(ctx, EV_SORT, EV_P2G);
            st.ms_prep = elapsed(ctx, EV_P2G, EV_PREP);
            st.ms_pcg_setup = elapsed(ctx, EV_PREP, EV_PCG_SETUP);
            st.ms_solve = elapsed(ctx, EV_PREP, EV_SOLVE);
            st.ms_extrapolate = elapsed(ctx, EV_SOLVE, EV_EXTRAP);
            st.ms_g2p = elapsed(ctx, EV_EXTRAP, EV_G2P);
            st.ms_g2p_kernel = st.ms_g2p;
            st.ms_total = elapsed(ctx, EV_START, EV_G2P);
        }
        *stats = st;
    }
    return FSIM_OK;
}

int fsim_get_grid(fsim_ctx* ctx, int field, void* out, int where) {
    if (!ctx || !out) return FSIM_E_INVALID;
    const GridGeom& g = ctx->g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    cudaStream_t s = ctx->stream;
    int elem = 4;
    void* dst = out;
    void* tmp = nullptr;
    if (field == FSIM_F_FLAGS) elem = 1;
    if (where == FSIM_HOST) {
        FSIM_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * elem, s));
        dst = tmp;
    }
    switch (field) {
        case FSIM_F_FLAGS: launch_pad_to_dense(g, ctx->flags, dst, 1, s); break;
        case FSIM_F_AVGPNUM: launch_pad_to_dense(g, ctx->avg, dst, 4, s); break;
        case FSIM_F_VX: case FSIM_F_VY: case FSIM_F_VZ:
            launch_pad_to_dense(g, ctx->u[field - FSIM_F_VX], dst, 4, s);
            break;
        case FSIM_F_V2X: case FSIM_F_V2Y: case FSIM_F_V2Z:
            launch_pad_to_dense(g, ctx->v2[field - FSIM_F_V2X], dst, 4, s);
            break;
        case FSIM_F_PRESSURE: launch_copy_phi(g, ctx->sv.phi, (float*)dst, s); break;
        case FSIM_F_COUNT: launch_counts(g, ctx->cstart, (int*)dst, s); break;
        case FSIM_F_DIVERGENCE: launch_rhs_out(ctx, (float*)dst); break;
        default:
            if (tmp) cudaFreeAsync(tmp, s);
            return set_error(ctx, FSIM_E_INVALID, "field id");
    }
    CHECK_LAUNCH(ctx);
    if (where == FSIM_HOST) {
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(out, tmp, (size_t)n * elem, cudaMemcpyDeviceToHost, s));
        FSIM_CUDA_TRY(ctx, cudaFreeAsync(tmp, s));
    }
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return FSIM_OK;
}

int fsim_set_grid(fsim_ctx* ctx, int field, const void* in, int where) {
    if (!ctx || !in) return FSIM_E_INVALID;
    const GridGeom& g = ctx->g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    cudaStream_t s = ctx->stream;
    const int elem = (field == FSIM_F_FLAGS) ? 1 : 4;
    const void* src = in;
    void* tmp = nullptr;
    if (where == FSIM_HOST) {
        FSIM_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * elem, s));
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(tmp, in, (size_t)n * elem, cudaMemcpyHostToDevice, s));
        src = tmp;
    }
    switch (field) {
        case FSIM_F_FLAGS: launch_dense_to_pad(g, src, ctx->flags, 1, s); break;
        case FSIM_F_AVGPNUM: launch_dense_to_pad(g, src, ctx->avg, 4, s); break;
        case FSIM_F_VX: case FSIM_F_VY: case FSIM_F_VZ:
            launch_dense_to_pad(g, src, ctx->u[field - FSIM_F_VX], 4, s);
            break;
        case FSIM_F_V2X: case FSIM_F_V2Y: case FSIM_F_V2Z:
            launch_dense_to_pad(g, src, ctx->v2[field - FSIM_F_V2X], 4, s);
            break;
        case FSIM_F_PRESSURE:
            k_dense_f32_to_f64_pad<<<ceil_div(n, 256), 256, 0, s>>>(g, (const float*)src, ctx->sv.phi);
            break;
        default:
            if (tmp) cudaFreeAsync(tmp, s);
            return set_error(ctx, FSIM_E_INVALID, "field id");
    }
    CHECK_LAUNCH(ctx);
    if (tmp) FSIM_CUDA_TRY(ctx, cudaFreeAsync(tmp, s));
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return FSIM_OK;
}

int fsim_fill_gfx_async(fsim_ctx* ctx, fsim_particle_gfx* out, int64_t cap, int64_t* n_out) {
    if (!ctx) return FSIM_E_INVALID;
    const long long n = ctx->n;
    if (n_out) *n_out = n;
    if (n == 0 || !out) return FSIM_OK;
    if (cap < n) return set_error(ctx, FSIM_E_INVALID, "output capacity below particle count");
    if (!ctx->copy_stream) {
        FSIM_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            FSIM_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->gfx_ready[k], cudaEventDisableTiming));
            FSIM_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->gfx_done[k], cudaEventDisableTiming));
            FSIM_CUDA_TRY(ctx, cudaEventRecord(ctx->gfx_done[k], ctx->copy_stream));
        }
    }
    const int k = ctx->gfx_slot;
    // the copy out of this slot (two hand-offs ago) must finish before it is rewritten
    FSIM_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->gfx_done[k], 0));
    if (ctx->gfx_cap[k] < n) {
        FSIM_CUDA_TRY(ctx, cudaEventSynchronize(ctx->gfx_done[k]));
        cudaFree(ctx->gfx_stage[k]);
        ctx->gfx_stage[k] = nullptr;
        ctx->gfx_cap[k] = 0;
        const long long c = n + n / 8 + 4096;
        if (cudaMalloc(&ctx->gfx_stage[k], (size_t)c * sizeof(fsim_particle_gfx)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(ctx, FSIM_E_OOM, "gfx staging buffer");
        }
        ctx->gfx_cap[k] = c;
    }
    launch_gfx(ctx->buf[ctx->cur], n, ctx->avg, ctx->g, ctx->gfx_stage[k], ctx->stream);
    ctx->launches += 1;
    CHECK_LAUNCH(ctx);
    FSIM_CUDA_TRY(ctx, cudaEventRecord(ctx->gfx_ready[k], ctx->stream));
    FSIM_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->gfx_ready[k], 0));
    FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->gfx_stage[k], (size_t)n * sizeof(fsim_particle_gfx),
                                       cudaMemcpyDeviceToHost, ctx->copy_stream));
    FSIM_CUDA_TRY(ctx, cudaEventRecord(ctx->gfx_done[k], ctx->copy_stream));
    ctx->gfx_slot = 1 - k;
    return FSIM_OK;
}

int fsim_gfx_wait(fsim_ctx* ctx) {
    if (!ctx) return FSIM_E_INVALID;
    if (ctx->copy_stream) FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->copy_stream));
    return FSIM_OK;
}

int fsim_fill_gfx(fsim_ctx* ctx, fsim_particle_gfx* out, int64_t cap, int64_t* n_out, int where) {
    if (!ctx) return FSIM_E_INVALID;
    const long long n = ctx->n;
    if (n_out) *n_out = n;
    if (n == 0 || !out) return FSIM_OK;
    if (cap < n) return set_error(ctx, FSIM_E_INVALID, "output capacity below particle count");
    cudaStream_t s = ctx->stream;
    fsim_particle_gfx* dst = out;
    void* tmp = nullptr;
    if (where == FSIM_HOST) {
        // Write straight into host memory when the GPU can address it: pinned or
        // registered buffers through their device alias, any host buffer on
        // systems with coherent access to pageable memory (NVLink-C2C hosts).
        cudaPointerAttributes attr{};
        void* alias = nullptr;
        int pageable = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, ctx->device);
        if (cudaPointerGetAttributes(&attr, out) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
            attr.devicePointer != nullptr) {
            alias = attr.devicePointer;
        } else if (pageable) {
            alias = out;
        }
        cudaGetLastError();
        if (alias) {
            dst = (fsim_particle_gfx*)alias;
        } else {
            FSIM_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * sizeof(fsim_particle_gfx), s));
            dst = (fsim_particle_gfx*)tmp;
        }
    }
    launch_gfx(ctx->buf[ctx->cur], n, ctx->avg, ctx->g, dst, s);
    ctx->launches += 1;
    CHECK_LAUNCH(ctx);
    if (tmp) {
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(out, tmp, (size_t)n * sizeof(fsim_particle_gfx), cudaMemcpyDeviceToHost, s));
        FSIM_CUDA_TRY(ctx, cudaFreeAsync(tmp, s));
    }
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return FSIM_OK;
}

int fsim_set_pressure_guess(fsim_ctx* ctx, const float* p, int where) {
    if (!ctx || !p) return FSIM_E_INVALID;
    const GridGeom& g = ctx->g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    cudaStream_t s = ctx->stream;
    const void* src = p;
    void* tmp = nullptr;
    if (where == FSIM_HOST) {
        FSIM_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * 4, s));
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(tmp, p, (size_t)n * 4, cudaMemcpyHostToDevice, s));
        src = tmp;
    }
    launch_dense_to_pad(g, src, ctx->sv.guess, 4, s);
    CHECK_LAUNCH(ctx);
    if (tmp) FSIM_CUDA_TRY(ctx, cudaFreeAsync(tmp, s));
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    ctx->sv.have_guess = true;
    return FSIM_OK;
}

int fsim_solve_current(fsim_ctx* ctx, double dt, int warm_start, int apply, fsim_step_stats* stats) {
    if (!ctx || !(dt > 0) || warm_start < FSIM_WARM_ZERO || warm_start > FSIM_WARM_LEARNED_RESIDUAL)
        return FSIM_E_INVALID;
    const fsim_params& P = ctx->prm;
    cudaStream_t s = ctx->stream;
    fsim_step_stats tmp{};
    fsim_step_stats* sp = stats ? stats : &tmp;
    const long long l0 = ctx->launches;
    FSIM_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[EV_PREP], s));
    int rc = solve_pressure(ctx, dt, P.precision, P.tol_mode, P.residual_tol, P.max_iters, warm_start, sp, nullptr,
                            apply);
    FSIM_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[EV_SOLVE], s));
    FSIM_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev[EV_SOLVE]));
    if (rc == FSIM_OK) {
        sp->ms_solve = elapsed(ctx, EV_PREP, EV_SOLVE);
        sp->kernel_launches = (int)(ctx->launches - l0);
        rc = check_device_error(ctx);
    }
    return rc;
}

int fsim_set_net(fsim_ctx* ctx, fsim_net* net) {
    if (!ctx) return FSIM_E_INVALID;
    ctx->net = net;
    return FSIM_OK;
}

int fsim_solve_pressure(fsim_ctx* ctx, const double* rhs, double dt, int precision, int tol_mode, double tol,
                        int max_iters, double* p_out, fsim_step_stats* stats) {
    if (!ctx || !rhs || !(dt > 0)) return FSIM_E_INVALID;
    const GridGeom& g = ctx->g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    cudaStream_t s = ctx->stream;
    const double scale = dt / (ctx->prm.fluid_density * g.hd * g.hd);
    std::vector<double> hb((size_t)n);
    for (long long j = 0; j < n; j++) hb[j] = rhs[j] / scale;
    double *dtmp = nullptr, *dpad = nullptr;
    FSIM_CUDA_TRY(ctx, cudaMallocAsync(&dtmp, (size_t)n * 8, s));
    FSIM_CUDA_TRY(ctx, cudaMallocAsync(&dpad, (size_t)g.ncell * 8, s));
    FSIM_CUDA_TRY(ctx, cudaMemsetAsync(dpad, 0, (size_t)g.ncell * 8, s));
    FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(dtmp, hb.data(), (size_t)n * 8, cudaMemcpyHostToDevice, s));
    launch_dense_to_pad(g, dtmp, dpad, 8, s);
    fsim_step_stats tmp{};
    fsim_step_stats* sp = stats ? stats : &tmp;
    cudaEventRecord(ctx->ev[EV_PREP], s);
    // zero start as the reference, or the judged learned guess when that is the configured warm start
    const int warm = ctx->prm.warm_start == FSIM_WARM_LEARNED ? FSIM_WARM_LEARNED : FSIM_WARM_ZERO;
    int rc = solve_pressure(ctx, dt, precision, tol_mode, tol, max_iters, warm, sp, dpad, 0);
    cudaEventRecord(ctx->ev[EV_SOLVE], s);
    cudaEventSynchronize(ctx->ev[EV_SOLVE]);
    if (rc == FSIM_OK) sp->ms_solve = elapsed(ctx, EV_PREP, EV_SOLVE);
    if (rc == FSIM_OK && p_out) {
        launch_pad_to_dense(g, ctx->sv.phi, dtmp, 8, s);
        cudaMemcpyAsync(p_out, dtmp, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
    }
    cudaFreeAsync(dtmp, s);
    cudaFreeAsync(dpad, s);
    FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return rc;
}

}  // extern "C"
