// fsim_ctx.h -- host-side context of the step library and the launchers each
// kernel translation unit exports to the orchestration in fsim_api.cu.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fsim_common.cuh"

// Pressure-solver state that lives on the device (scalars of PCG in FP64).
struct PcgState {
    double sigma;        // z.r
    double sigma_prev;   // z.r of the previous iteration (for reliable updates)
    double alpha, beta;
    double rmax, rr;     // recursive residual max |r|, r.r   (A' units)
    double rr_update;    // r.r right after the last true-residual replacement
    double fold_drop;    // MIXED: fold + restart once r.r < fold_drop * rr_update
    double bb, bmax;     // rhs norms (A' units)
    double tol_abs;      // max-norm tolerance in A' units
    double tol_rel2;     // (tol * ||b||)^2 in A' units
    int tol_mode;
    int it;              // iterations done
    int max_iters;
    int done;            // 1 = stop iterating (converged candidate or iteration cap or NaN)
    int converged;       // recursive residual met the tolerance
    int nan;
    int skip;            // rhs below the reference's early-out (sum b^2 < 1e-7)
    int bufsel;          // bit 0: current r buffer, bit 1: current s buffer
    int fold_enabled;    // MIXED: stop the inner iteration when r.r fell by fold_drop
    int need_fold;       // set by the iteration when a fold + restart is due
    int guess_used;      // the judged guess had the smaller residual and seeds PCG
};

// One level of the multigrid hierarchy (level 0 is the simulation grid).
struct MGLevelBufs {
    int nx = 0, ny = 0, nz = 0, pz = 0;
    long long ncell = 0;          // nx * ny * pz
    uint8_t* kind = nullptr;      // 0 fluid, 1 air, 2 solid (levels >= 1)
    uint16_t* code = nullptr;     // same encoding as SolverBufs::code
    float* x = nullptr;           // correction (levels >= 1)
    float* f = nullptr;           // right-hand side (levels >= 1)
    float* r = nullptr;           // residual
};

struct SolverBufs {
    double conv_rate[2] = {0.0, 0.0};  // measured PCG residual-norm factor per iteration, per
                                       // preconditioner (RB-IC, multigrid): chunk planning
    int nbx, nby, nbz;         // bricks per axis
    long long nbricks;
    int4* brick_xyz = nullptr; // active bricks (contain a fluid cell), ascending: {bx, by, bz, b}
    int* d_nactive = nullptr;  // device count of active bricks
    uint8_t* brick_flag = nullptr;
    uint16_t* code = nullptr;  // per cell: fluid-neighbour mask, non-solid count, self fluid
    double* b = nullptr;       // rhs in A' units (A' = A / scale: integer 7-point stencil)
    double* phi = nullptr;     // FP64 solution (pressure)
    // FP32 Krylov vectors (MIXED / FP32)
    float *r = nullptr, *z = nullptr, *s = nullptr, *q = nullptr, *plo = nullptr;
    // FP64 Krylov vectors (FP64 precision)
    double *r64 = nullptr, *z64 = nullptr, *s64 = nullptr, *q64 = nullptr;
    double* partials = nullptr;
    unsigned* counter = nullptr;
    PcgState* st = nullptr;       // device
    PcgState* st_host = nullptr;  // pinned mirror
    float* guess = nullptr;       // user / learned initial guess (reference order packed)
    bool have_guess = false;
    int grid_blocks = 0;          // persistent grid size for brick kernels
    double last_scale = 1.0;      // dt / (rho h^2) of the last solve
    std::vector<MGLevelBufs> mg;  // multigrid hierarchy (built at allocation)
    int mg_cluster = 0;           // CTAs in the coarse-V-cycle cluster (0: separate launches)
    int4* bnd_quads = nullptr;    // finest-level quads of the free-surface band {x, y, z0, 0}
    int* d_nbnd = nullptr;        // their count (device)
    // one PCG iteration as a CUDA graph, captured on first use per configuration
    // (precision, preconditioner, sweep counts); up to four are kept
    static constexpr int kIterGraphs = 4;
    cudaGraphExec_t iter_exec[kIterGraphs] = {};
    int iter_key[kIterGraphs] = {-1, -1, -1, -1};
    int iter_kernels[kIterGraphs] = {};
    long long iter_used[kIterGraphs] = {};  // last use (for replacement)
    long long iter_clock = 0;
};

struct fsim_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // asynchronous gfx hand-off (fsim_fill_gfx_async): double-buffered device
    // staging, copied to the host on copy_stream
    cudaStream_t copy_stream = nullptr;
    fsim_particle_gfx* gfx_stage[2] = {nullptr, nullptr};
    long long gfx_cap[2] = {0, 0};
    cudaEvent_t gfx_ready[2] = {nullptr, nullptr};
    cudaEvent_t gfx_done[2] = {nullptr, nullptr};
    int gfx_slot = 0;
    fsim_params prm{};
    GridGeom g{};
    std::string err;

    // particles
    long long n = 0, cap = 0;
    ParticleBuf buf[2]{};
    void* buf_mem[2] = {nullptr, nullptr};
    int cur = 0;
    uint32_t next_id = 0;
    uint32_t* key = nullptr;
    uint32_t* rank = nullptr;
    uint32_t* perm = nullptr;
    int* count = nullptr;   // ncell
    int* cstart = nullptr;  // ncell + 1
    int* scan_blocks = nullptr;
    bool sorted = false;    // perm/cstart describe the current buffer's positions
    long long n_sorted = 0;

    // grid (padded layout)
    uint8_t* flags = nullptr;
    float* u[3] = {nullptr, nullptr, nullptr};   // face v
    float* v2[3] = {nullptr, nullptr, nullptr};  // face v2
    float* avg = nullptr;
    uint8_t* valid = nullptr;

    SolverBufs sv;

    // obstacles (host copy; sources carry last_spawn_fraction)
    std::vector<fsim_obstacle> obs;
    uint64_t spawn_counter = 0;
    // disc-source cell lists of a step: mapped pinned host memory the spawn
    // kernel reads directly (no copy-engine transfer inside a step)
    int* disc_cells_host = nullptr;
    int* disc_cells_dev = nullptr;
    long long disc_cells_cap = 0;

    // TMA descriptors for the G2P tile loads (v2 x/y/z, v x/y/z)
    CUtensorMap tmap[6];
    bool tmap_ok = false;

    // device error word + pinned mirrors
    unsigned* d_err = nullptr;
    int* d_misc = nullptr;   // small device scratch (counts)
    int* h_misc = nullptr;   // pinned

    fsim_net* net = nullptr;  // warm-start network (FSIM_WARM_LEARNED), not owned
    int learned_skip = 0;     // solves left before the network is judged again (learned_backoff)
    int learned_wait = 0;     // the current back-off length

    cudaEvent_t ev[16];
    bool events = false;
    long long launches = 0;  // kernels launched by this context (monotonic)
};

// ---- launchers (k_particles.cu) -------------------------------------------
struct AdvectArgs {
    ParticleBuf p;
    long long n;
    int do_advect, do_push, do_stop, do_key, despawn;
    int keep_dead;         // particles whose key is already DEAD stay dead (second pass of a step)
    float dt;
    float lo[3], hi[3];    // advection clamp band (gridLow / gridHigh)
    float plo[3], phi[3];  // push-out clamp band
    float pr;              // particle radius
    int nobs;
    DevObstacle obs[FSIM_MAX_OBS];
    GridGeom g;
    uint32_t* key;
    uint32_t* rank;
    int* count;
};
void launch_advect(const AdvectArgs& a, cudaStream_t s);
void launch_scan(const int* in, int* out, long long n, int* block_sums, cudaStream_t s);
// perm[cstart[key] + rank] = index, then each cell's segment in ascending
// particle index (two kernels when n > 0)
void launch_scatter(const uint32_t* key, const uint32_t* rank, const int* cstart, uint32_t* perm,
                    long long n, long long ncell, cudaStream_t s);
void launch_gather(ParticleBuf src, ParticleBuf dst, const uint32_t* perm, const int* cstart,
                   long long ncell, long long n, bool ids, cudaStream_t s);
void launch_spawn_sphere(ParticleBuf p, long long first, int count, const fsim_obstacle& o,
                         double particle_r, uint64_t seed, uint32_t first_id, bool ids,
                         cudaStream_t s);
void launch_spawn_disc(ParticleBuf p, long long first, int ncells, const fsim_obstacle& o,
                       const GridGeom& g, int cy, const int* cells_xz, uint64_t seed,
                       uint32_t first_id, bool ids, cudaStream_t s);
void launch_push_apart(ParticleBuf p, const uint32_t* perm, const int* cstart, const GridGeom& g, long long n,
                       double r, const float lo[3], const float hi[3], float* const out[3], cudaStream_t s);
// Small device -> pinned-host reads (solver state, counts, error flags) by a
// one-warp kernel writing through the host mapping instead of a DMA copy, so
// that they never queue behind a large copy-engine transfer (the asynchronous
// gfx hand-off).  `host` must be cudaMallocHost memory; valid after a
// synchronize of `s`.
void fetch_small(void* host, const void* dev, int bytes, cudaStream_t s);
void launch_gfx(ParticleBuf p, long long n, const float* avg, const GridGeom& g,
                fsim_particle_gfx* out, cudaStream_t s);

// ---- launchers (k_transfer.cu) ---------------------------------------------
void launch_p2g(fsim_ctx* ctx);
int launch_g2p(fsim_ctx* ctx);
bool make_tensor_maps(fsim_ctx* ctx);
// Returns the launch's error (a failed shared-memory attribute set included).
cudaError_t launch_p2g_raw(ParticleBuf p, const uint32_t* perm, const int* cstart, const GridGeom& g,
                           float* const u[3], uint8_t* flags, float* avg, bool apic, cudaStream_t stream);

// ---- launchers (k_grid.cu) -------------------------------------------------
int launch_obstacle(fsim_ctx* ctx, const fsim_obstacle& o);  // returns kernels launched
void launch_prep(fsim_ctx* ctx, int walls, int post, float gravity_inc);
void launch_extrapolate(fsim_ctx* ctx);
void launch_apply_pressure(fsim_ctx* ctx, double dt);
int launch_sor(fsim_ctx* ctx, int iters);  // BasicMacGrid solver; returns the sweeps run
void launch_pad_to_dense(const GridGeom& g, const void* src, void* dst, int elem, cudaStream_t s);
void launch_dense_to_pad(const GridGeom& g, const void* src, void* dst, int elem, cudaStream_t s);
void launch_counts(const GridGeom& g, const int* cstart, int* out, cudaStream_t s);
void launch_copy_phi(const GridGeom& g, const double* phi, float* out, cudaStream_t s);
void launch_rhs_out(fsim_ctx* ctx, float* out);

// ---- launchers (k_pcg.cu) --------------------------------------------------
int solver_alloc(fsim_ctx* ctx);
void solver_free(fsim_ctx* ctx);
// Run the pressure solve on the current flags / v2 and apply it to v2.
// rhs_override: rhs in A' units (padded layout) instead of the divergence of v2;
// apply: add the pressure gradient to v2 afterwards.
int solve_pressure(fsim_ctx* ctx, double dt, int precision, int tol_mode, double tol,
                   int max_iters, int warm, fsim_step_stats* st, const double* rhs_override, int apply);

// Event slots of a step (recorded when fsim_params.timing is set).
enum {
    EV_START = 0, EV_ADVECT, EV_SORT, EV_P2G, EV_PREP, EV_PCG_SETUP, EV_SOLVE, EV_EXTRAP, EV_G2P, EV_GUESS0,
    EV_GUESS1, EV_APART, EV_COUNT
};
inline void fsim_record(fsim_ctx* ctx, int k) {
    if (ctx->prm.timing) cudaEventRecord(ctx->ev[k], ctx->stream);
}

#define FSIM_CUDA_TRY(ctx, call)                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);       \
            return FSIM_E_CUDA;                                                    \
        }                                                                          \
    } while (0)
