// k_pcg.cu -- pressure projection: matrix-free preconditioned conjugate
// gradients on the MAC grid (replaces BridsonSolverGrid::solveIncompressibility,
// bridsonSolverGrid.cpp:244-293).
//
// System.  The reference assembles A with scale = dt/(rho h^2): diagonal =
// scale * (number of non-SOLID neighbours), off-diagonal = -scale towards fluid
// neighbours (calculateAMatrix, :40-77), and b = -(1/h) div(v2) [+ density
// term] (calculateRHS, :79-89).  Here the solver works on A' = A / scale, an
// integer 7-point stencil read straight from a 16-bit code per cell (fluid-
// neighbour mask + non-solid count), and b' = b / scale; the solution is the
// same p.  No matrix is stored.
//
// Preconditioner.  Incomplete Cholesky in red-black order (red = x+y+z even).
// Red rows have no earlier neighbours, so their pivots are the diagonal; a
// black pivot is d_B = ns_B - sum_j (1 + tau (nf_j - 1)) / ns_j over its red
// fluid neighbours j (the modified-IC fill compensation of the reference's
// MIC(0), tau = 0.97, with its safeguard d < 0.25 ns -> d = ns).  Applying M^-1
// is two half sweeps: z_B = (r_B + sum_j r_j / ns_j) / d_B, then
// z_R = (r_R + sum_k z_k) / ns_R; both colours are fully parallel.
//
// Precision (FSIM_PREC_MIXED).  Krylov vectors, stencil and preconditioner in
// FP32; dot products, alpha/beta and the convergence test in FP64; the
// solution accumulates in FP32 and is folded into an FP64 solution with the
// true residual b' - A' p recomputed in FP64 whenever the recursive residual
// has dropped by 10x since the last fold ("reliable updates"), and always
// before convergence is declared.  FSIM_PREC_FP32 never folds until the end;
// FSIM_PREC_FP64 runs every vector in FP64.
//
// Work layout.  Cells are grouped in 2x4x32 bricks (one 256-thread CTA pass
// per brick); only bricks holding a fluid cell are visited.  Per iteration
// three kernels: (1) s = z + beta s, q = A' s, s.q; (2) x += alpha s,
// r -= alpha q, black half-sweep, r.r / max|r|; (3) red half-sweep, z.r.
// Each reduction finishes in the last CTA to arrive (fixed order, so results
// are deterministic), which also updates the scalars in device memory; the
// host only polls a small state block every few iterations.
#include <cmath>

#include "fsim_ctx.h"

namespace {

constexpr int BRX = 2, BRY = 4, BRZ = 32;
constexpr int PCG_THREADS = 256;
constexpr float TAU = 0.97f;
constexpr float SAFE = 0.25f;

// code bits
constexpr uint16_t CODE_FLUID = 0x8000;
__device__ __forceinline__ int code_ns(uint16_t c) { return (c >> 8) & 7; }
__device__ __forceinline__ int code_nf(uint16_t c) { return __popc(c & 0x3F); }

struct BrickGeo {
    GridGeom g;
    int nbx, nby, nbz;
    long long sx, sy;  // strides of +x and +y (+z is 1)
};

// neighbour offset k: +x, -x, +y, -y, +z, -z (bit k of the fluid mask)
__device__ __forceinline__ long long nb_off(const BrickGeo& B, int k) {
    const long long st = (k >> 1) == 0 ? B.sx : ((k >> 1) == 1 ? B.sy : 1ll);
    return (k & 1) ? -st : st;
}

__device__ __forceinline__ bool brick_cell(const BrickGeo& B, int b, int t, int& x, int& y, int& z,
                                           long long& c) {
    const int bz = b % B.nbz, by = (b / B.nbz) % B.nby, bx = b / (B.nbz * B.nby);
    x = bx * BRX + t / (BRY * BRZ);
    y = by * BRY + (t / BRZ) % BRY;
    z = bz * BRZ + t % BRZ;
    if (x >= B.g.nx || y >= B.g.ny || z >= B.g.nz) return false;
    c = gidx(B.g, x, y, z);
    return true;
}

__constant__ float c_fill[7][7];  // (1 + tau (nf - 1)) / ns
__constant__ float c_rcp[7];      // 1 / ns (1 for ns = 0)

// Per-thread sums.  GB300 runs FP64 at a small fraction of its FP32 rate, so
// per-cell terms are summed in FP32 with compensation (Kahan), and only the
// per-thread totals enter the FP64 block / grid reduction.
template <typename T>
struct Acc {
    T s = 0;
    __device__ __forceinline__ void add(T x) { s += x; }
    __device__ __forceinline__ double value() const { return (double)s; }
};
template <>
struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <typename T>
__device__ __forceinline__ T recip_ns(int ns);
template <>
__device__ __forceinline__ float recip_ns<float>(int ns) { return c_rcp[ns]; }
template <>
__device__ __forceinline__ double recip_ns<double>(int ns) { return ns > 0 ? 1.0 / ns : 1.0; }

__device__ __forceinline__ float black_pivot_inv(const uint16_t* code, long long c, uint16_t cc,
                                                 const BrickGeo& B) {
    const int ns = code_ns(cc);
    if (ns == 0) return 1.f;
    float d = (float)ns;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        if ((cc >> k) & 1) {
            const uint16_t cj = code[c + nb_off(B, k)];
            d -= c_fill[code_nf(cj)][code_ns(cj)];
        }
    }
    if (d < SAFE * ns) d = (float)ns;
    return __frcp_rn(d);
}

// ---- setup: codes, rhs, initial guess, brick activity ----------------------
struct SetupArgs {
    BrickGeo B;
    const uint8_t* flags;
    const float* v2[3];
    const float* avg;
    const float* guess;   // padded layout, or null
    const double* rhs_override;  // padded layout in A' units, or null
    int warm;             // FSIM_WARM_*
    int pressure_enabled;
    double avg_pressure, pressure_k;
    double inv_h, inv_scale;
    uint16_t* code;
    double* b;
    double* phi;
    uint8_t* brick_flag;
};

__global__ void k_setup(const SetupArgs a) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const GridGeom& g = a.B.g;
    if (c >= g.ncell) return;
    const int z = (int)(c % g.pz);
    if (z >= g.nz) return;
    const int y = (int)((c / g.pz) % g.ny), x = (int)(c / ((long long)g.pz * g.ny));
    const uint8_t f = a.flags[c];
    if (f != C_WATER || x == 0 || y == 0 || z == 0 || x == g.nx - 1 || y == g.ny - 1 || z == g.nz - 1) {
        a.code[c] = 0;
        if (a.phi[c] != 0.0) a.phi[c] = 0.0;
        return;
    }
    uint16_t code = CODE_FLUID;
    int ns = 0;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const uint8_t fn = a.flags[c + nb_off(a.B, k)];
        if (fn == C_WATER) code |= (uint16_t)(1u << k);
        if (fn != C_SOLID) ns++;
    }
    code |= (uint16_t)(ns << 8);
    a.code[c] = code;
    double bb;
    if (a.rhs_override) {
        bb = a.rhs_override[c];
    } else {
        const double sum = (double)a.v2[0][c] + (double)a.v2[1][c] + (double)a.v2[2][c] -
                           (double)a.v2[0][c - a.B.sx] - (double)a.v2[1][c - a.B.sy] -
                           (double)a.v2[2][c - 1];
        double rhs = -a.inv_h * sum;
        if (a.pressure_enabled) rhs += ((double)a.avg[c] - a.avg_pressure) * a.pressure_k;
        bb = rhs * a.inv_scale;
    }
    a.b[c] = bb;
    if (a.warm == FSIM_WARM_ZERO) a.phi[c] = 0.0;
    else if (a.warm == FSIM_WARM_GUESS && a.guess) a.phi[c] = (double)a.guess[c];
    const int bz = z / BRZ, by = y / BRY, bx = x / BRX;
    a.brick_flag[((long long)bx * a.B.nby + by) * a.B.nbz + bz] = 1;
}

// ordered compaction of active bricks (one CTA)
__global__ void __launch_bounds__(1024) k_compact_bricks(const uint8_t* flag, long long nb, int* list,
                                                         int* count) {
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long base = 0; base < nb; base += blockDim.x) {
        const long long j = base + threadIdx.x;
        const int f = (j < nb) ? flag[j] : 0;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        int before = 0;
        for (int w = 0; w < warp; w++) before += warp_tot[w];
        if (f) list[carry + before + __popc(bal & ((1u << lane) - 1u))] = (int)j;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += warp_tot[w];
            carry += t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

struct PcgArgs {
    BrickGeo B;
    const int* list;
    const int* nactive;
    const uint16_t* code;
    const double* b;
    double* phi;
    PcgState* st;
    double* partials;
    unsigned* counter;
    double tol_abs, tol_rel;  // tolerance in A' units (abs) / relative
    double skip_bb;           // early-out threshold on b'.b' (reference: sum b^2 < 1e-7)
};

template <typename T>
struct Vecs {
    T* r[2];
    T* s[2];
    T* z;
    T* q;
    T* x;  // accumulated solution (float plo for FP32/MIXED, double phi for FP64)
};

// r = b' - A' phi (FP64), store into r[rc]; reset x (FP32 accumulator) to 0.
// first = 1: also reduce |b'| and decide the reference's early-out.
template <typename T>
__global__ void __launch_bounds__(PCG_THREADS) k_residual(const PcgArgs a, Vecs<T> v, int first, int reset_x) {
    __shared__ double scratch[32 * 4];
    T* r = (a.st->bufsel & 1) ? v.r[1] : v.r[0];
    double acc[4] = {0.0, -1e300, 0.0, -1e300};  // rr, rmax, bb, bmax
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.list[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        const double* phi = a.phi;
        double ap = (double)code_ns(cc) * phi[c];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if ((cc >> k) & 1) ap -= phi[c + nb_off(a.B, k)];
        const double bc = a.b[c];
        const double rv = bc - ap;
        r[c] = (T)rv;
        if (reset_x && sizeof(T) == 4) v.x[c] = (T)0;
        acc[0] += rv * rv;
        acc[1] = fmax(acc[1], fabs(rv));
        acc[2] += bc * bc;
        acc[3] = fmax(acc[3], fabs(bc));
    }
    if (last_block_reduce<4>(acc, 0xA, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* s = a.st;
            s->rr = acc[0];
            s->rmax = acc[1];
            s->rr_update = acc[0];
            if (first) {
                s->bb = acc[2];
                s->bmax = acc[3];
                s->tol_rel2 = a.tol_rel * a.tol_rel * acc[2];
                s->skip = acc[2] < a.skip_bb ? 1 : 0;
            }
            const bool conv = (s->tol_mode == FSIM_TOL_ABS_MAX) ? (acc[1] < a.tol_abs) : (acc[0] <= s->tol_rel2);
            s->converged = conv ? 1 : 0;
            s->done = (conv || s->skip) ? 1 : 0;
        }
    }
}

// black half-sweep from r[rc] (setup / after a fold)
template <typename T>
__global__ void __launch_bounds__(PCG_THREADS) k_black(const PcgArgs a, Vecs<T> v) {
    if (a.st->done) return;
    const int rc = a.st->bufsel & 1;
    const T* r = rc ? v.r[1] : v.r[0];
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.list[bk], threadIdx.x, x, y, z, c)) continue;
        if (((x + y + z) & 1) == 0) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        T sum = r[c];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if ((cc >> k) & 1) {
                const long long j = c + nb_off(a.B, k);
                sum += r[j] * recip_ns<T>(code_ns(a.code[j]));
            }
        v.z[c] = sum * (T)black_pivot_inv(a.code, c, cc, a.B);
    }
}

// red half-sweep + z.r over all fluid cells.
// mode 0: sigma = z.r, beta = 0 (setup)
// mode 1: beta = z.r / sigma, sigma_prev = sigma, sigma = z.r   (iteration)
// mode 2: beta = z.r / sigma_prev, sigma = z.r                  (after a fold)
template <typename T>
__global__ void __launch_bounds__(PCG_THREADS) k_red(const PcgArgs a, Vecs<T> v, int mode) {
    __shared__ double scratch[32];
    if (a.st->done) return;
    const int rc = a.st->bufsel & 1;
    const T* r = rc ? v.r[1] : v.r[0];
    Acc<T> zr;
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.list[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        const T rv = r[c];
        T zv;
        if (((x + y + z) & 1) == 0) {
            T sum = rv;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if ((cc >> k) & 1) sum += v.z[c + nb_off(a.B, k)];
            zv = sum * recip_ns<T>(code_ns(cc));
            v.z[c] = zv;
        } else {
            zv = v.z[c];
        }
        zr.add(zv * rv);
    }
    double acc[1] = {zr.value()};
    if (last_block_reduce<1>(acc, 0, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* s = a.st;
            const double sig = acc[0];
            if (mode == 0) {
                s->beta = 0.0;
                s->sigma = sig;
                s->sigma_prev = sig;
            } else if (mode == 1) {
                s->beta = sig / s->sigma;
                s->sigma_prev = s->sigma;
                s->sigma = sig;
            } else {
                s->beta = sig / s->sigma_prev;
                s->sigma = sig;
            }
            if (!isfinite(s->beta)) {
                s->nan = 1;
                s->done = 1;
            }
        }
    }
}

// s_new = z + beta s_old; q = A' s_new; alpha = sigma / (s.q)
template <typename T>
__global__ void __launch_bounds__(PCG_THREADS) k_spmv(const PcgArgs a, Vecs<T> v) {
    __shared__ double scratch[32];
    if (a.st->done) return;
    const int sc = (a.st->bufsel >> 1) & 1;
    const double beta = a.st->beta;
    const T* so = sc ? v.s[1] : v.s[0];
    T* sn = sc ? v.s[0] : v.s[1];
    Acc<T> sq;
    const T betaT = (T)beta;
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.list[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        const T snc = v.z[c] + betaT * so[c];
        T qv = (T)code_ns(cc) * snc;
#pragma unroll
        for (int k = 0; k < 6; k++)
            if ((cc >> k) & 1) {
                const long long j = c + nb_off(a.B, k);
                qv -= v.z[j] + betaT * so[j];
            }
        sn[c] = snc;
        v.q[c] = qv;
        sq.add(snc * qv);
    }
    double acc[1] = {sq.value()};
    if (last_block_reduce<1>(acc, 0, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* s = a.st;
            s->alpha = s->sigma / acc[0];
            if (!isfinite(s->alpha)) {
                s->nan = 1;
                s->done = 1;
            }
            s->bufsel ^= 2;  // s buffers swap
        }
    }
}

// x += alpha s; r_new = r - alpha q; black half-sweep on r_new; r.r, max|r|
template <typename T>
__global__ void __launch_bounds__(PCG_THREADS) k_update(const PcgArgs a, Vecs<T> v) {
    __shared__ double scratch[32 * 2];
    if (a.st->done) return;
    const int rc = a.st->bufsel & 1, sc = (a.st->bufsel >> 1) & 1;
    const T alpha = (T)a.st->alpha;
    const T* ro = rc ? v.r[1] : v.r[0];
    T* rn = rc ? v.r[0] : v.r[1];
    const T* s = sc ? v.s[1] : v.s[0];
    Acc<T> rr;
    T rmax = (T)0;
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.list[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        v.x[c] += alpha * s[c];
        const T rv = ro[c] - alpha * v.q[c];
        rn[c] = rv;
        rr.add(rv * rv);
        rmax = fmax(rmax, fabs(rv));
        if ((x + y + z) & 1) {
            T sum = rv;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if ((cc >> k) & 1) {
                    const long long j = c + nb_off(a.B, k);
                    const uint16_t cj = a.code[j];
                    sum += (ro[j] - alpha * v.q[j]) * recip_ns<T>(code_ns(cj));
                }
            v.z[c] = sum * (T)black_pivot_inv(a.code, c, cc, a.B);
        }
    }
    double acc[2] = {rr.value(), (double)rmax};
    if (last_block_reduce<2>(acc, 0x2, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* st = a.st;
            st->rr = acc[0];
            st->rmax = acc[1];
            st->it += 1;
            st->bufsel ^= 1;  // r buffers swap
            const bool conv = (st->tol_mode == FSIM_TOL_ABS_MAX) ? (acc[1] < a.tol_abs) : (acc[0] <= st->tol_rel2);
            st->converged = conv ? 1 : 0;
            if (conv || st->it >= st->max_iters || !isfinite(acc[0])) st->done = 1;
            if (!isfinite(acc[0])) st->nan = 1;
        }
    }
}

// phi += x; x = 0   (fold the FP32 accumulator into the FP64 solution)
__global__ void __launch_bounds__(PCG_THREADS) k_fold(const PcgArgs a, float* x) {
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int xx, y, z;
        long long c;
        if (!brick_cell(a.B, a.list[bk], threadIdx.x, xx, y, z, c)) continue;
        if (!(a.code[c] & CODE_FLUID)) continue;
        a.phi[c] += (double)x[c];
        x[c] = 0.f;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int solver_alloc(fsim_ctx* ctx) {
    SolverBufs& S = ctx->sv;
    const GridGeom& g = ctx->g;
    S.nbx = ceil_div(g.nx, BRX);
    S.nby = ceil_div(g.ny, BRY);
    S.nbz = ceil_div(g.nz, BRZ);
    S.nbricks = (long long)S.nbx * S.nby * S.nbz;
    const size_t nc = (size_t)g.ncell;
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.brick_list, S.nbricks * sizeof(int)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.d_nactive, sizeof(int)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.brick_flag, S.nbricks));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.code, nc * sizeof(uint16_t)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.b, nc * sizeof(double)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.phi, nc * sizeof(double)));
    FSIM_CUDA_TRY(ctx, cudaMemset(S.phi, 0, nc * sizeof(double)));
    // FP32 set: r[2], s[2], z, q, x  (7 arrays, one allocation)
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.r, 7 * nc * sizeof(float)));
    FSIM_CUDA_TRY(ctx, cudaMemset(S.r, 0, 7 * nc * sizeof(float)));
    S.s = S.r + 2 * nc;
    S.z = S.r + 4 * nc;
    S.q = S.r + 5 * nc;
    S.plo = S.r + 6 * nc;
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_update<float>, PCG_THREADS, 0);
    if (bps < 1) bps = 1;
    S.grid_blocks = ctx->num_sms * bps;
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.partials, (size_t)S.grid_blocks * 4 * sizeof(double)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.counter, sizeof(unsigned)));
    FSIM_CUDA_TRY(ctx, cudaMemset(S.counter, 0, sizeof(unsigned)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.st, sizeof(PcgState)));
    FSIM_CUDA_TRY(ctx, cudaMallocHost(&S.st_host, sizeof(PcgState)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.guess, nc * sizeof(float)));
    float fill[7][7];
    for (int nf = 0; nf < 7; nf++)
        for (int ns = 0; ns < 7; ns++) fill[nf][ns] = ns > 0 ? (1.f + TAU * (nf - 1)) / ns : 0.f;
    FSIM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_fill, fill, sizeof(fill)));
    float rcp[7];
    for (int ns = 0; ns < 7; ns++) rcp[ns] = ns > 0 ? 1.f / ns : 1.f;
    FSIM_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_rcp, rcp, sizeof(rcp)));
    return FSIM_OK;
}

static int alloc_fp64(fsim_ctx* ctx) {
    SolverBufs& S = ctx->sv;
    if (S.r64) return FSIM_OK;
    const size_t nc = (size_t)ctx->g.ncell;
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.r64, 6 * nc * sizeof(double)));
    FSIM_CUDA_TRY(ctx, cudaMemset(S.r64, 0, 6 * nc * sizeof(double)));
    S.s64 = S.r64 + 2 * nc;
    S.z64 = S.r64 + 4 * nc;
    S.q64 = S.r64 + 5 * nc;
    return FSIM_OK;
}

void solver_free(fsim_ctx* ctx) {
    SolverBufs& S = ctx->sv;
    cudaFree(S.brick_list); cudaFree(S.d_nactive); cudaFree(S.brick_flag); cudaFree(S.code);
    cudaFree(S.b); cudaFree(S.phi); cudaFree(S.r); cudaFree(S.r64); cudaFree(S.partials);
    cudaFree(S.counter); cudaFree(S.st); cudaFreeHost(S.st_host); cudaFree(S.guess);
    S = SolverBufs{};
}

template <typename T>
static int run_pcg(fsim_ctx* ctx, PcgArgs& A, Vecs<T> v, int precision, fsim_step_stats* stats) {
    SolverBufs& S = ctx->sv;
    cudaStream_t st = ctx->stream;
    const int G = S.grid_blocks;
    const bool fold = (precision == FSIM_PREC_MIXED);
    int folds = 0;
    auto read_state = [&]() -> int {
        FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(S.st_host, S.st, sizeof(PcgState), cudaMemcpyDeviceToHost, st));
        FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        return FSIM_OK;
    };
    // initial residual, preconditioned residual, sigma
    k_residual<T><<<G, PCG_THREADS, 0, st>>>(A, v, 1, 1);
    k_black<T><<<G, PCG_THREADS, 0, st>>>(A, v);
    k_red<T><<<G, PCG_THREADS, 0, st>>>(A, v, 0);
    ctx->launches += 3;
    fsim_record(ctx, EV_PCG_SETUP);
    int rc = read_state();
    if (rc) return rc;
    int chunk = 4;
    while (!S.st_host->done && !S.st_host->nan) {
        for (int k = 0; k < chunk; k++) {
            k_spmv<T><<<G, PCG_THREADS, 0, st>>>(A, v);
            k_update<T><<<G, PCG_THREADS, 0, st>>>(A, v);
            k_red<T><<<G, PCG_THREADS, 0, st>>>(A, v, 1);
        }
        ctx->launches += 3 * chunk;
        if ((rc = read_state())) return rc;
        if (chunk < 16) chunk *= 2;
        PcgState& h = *S.st_host;
        if (h.nan) break;
        const bool need_fold = fold && (h.done || h.rr < 0.01 * h.rr_update);
        if (need_fold && !h.skip) {
            // fold, recompute the true residual in FP64, restart the preconditioned residual
            k_fold<<<G, PCG_THREADS, 0, st>>>(A, (float*)(void*)v.x);
            const int it_before = h.it;
            const int was_done = h.done;
            h.done = 0;
            FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(&S.st->done, &h.done, sizeof(int), cudaMemcpyHostToDevice, st));
            k_residual<T><<<G, PCG_THREADS, 0, st>>>(A, v, 0, 0);
            k_black<T><<<G, PCG_THREADS, 0, st>>>(A, v);
            k_red<T><<<G, PCG_THREADS, 0, st>>>(A, v, 2);
            ctx->launches += 4;
            folds++;
            if ((rc = read_state())) return rc;
            if (!h.done && it_before >= h.max_iters) {
                h.done = 1;
            }
            (void)was_done;
            if (h.done) break;
        } else if (h.done) {
            break;
        }
    }
    if (precision == FSIM_PREC_FP32) {
        k_fold<<<G, PCG_THREADS, 0, st>>>(A, (float*)(void*)v.x);
        ctx->launches += 2;
        // true residual of the FP32 result (reporting only)
        PcgState& h = *S.st_host;
        const int conv_recursive = h.converged, its = h.it;
        k_residual<T><<<G, PCG_THREADS, 0, st>>>(A, v, 0, 0);
        if ((rc = read_state())) return rc;
        h.it = its;
        h.converged = conv_recursive;
    }
    if (stats) {
        PcgState& h = *S.st_host;
        stats->pcg_iterations = h.it;
        stats->converged = h.converged;
        stats->reliable_updates = folds;
    }
    return FSIM_OK;
}

int solve_pressure(fsim_ctx* ctx, double dt, int precision, int tol_mode, double tol, int max_iters,
                   int warm, fsim_step_stats* stats, const double* rhs_override, int apply) {
    SolverBufs& S = ctx->sv;
    const GridGeom& g = ctx->g;
    cudaStream_t st = ctx->stream;
    const double scale = dt / (ctx->prm.fluid_density * g.hd * g.hd);
    S.last_scale = scale;
    BrickGeo B;
    B.g = g;
    B.nbx = S.nbx; B.nby = S.nby; B.nbz = S.nbz;
    B.sx = (long long)g.pz * g.ny;
    B.sy = g.pz;

    FSIM_CUDA_TRY(ctx, cudaMemsetAsync(S.brick_flag, 0, S.nbricks, st));
    SetupArgs sa;
    sa.B = B;
    sa.flags = ctx->flags;
    for (int a = 0; a < 3; a++) sa.v2[a] = ctx->v2[a];
    sa.avg = ctx->avg;
    sa.guess = (warm == FSIM_WARM_GUESS && S.have_guess) ? S.guess : nullptr;
    sa.rhs_override = rhs_override;
    sa.warm = warm;
    sa.pressure_enabled = ctx->prm.pressure_enabled;
    sa.avg_pressure = ctx->prm.average_pressure;
    sa.pressure_k = ctx->prm.pressure_k;
    sa.inv_h = 1.0 / g.hd;
    sa.inv_scale = 1.0 / scale;
    sa.code = S.code;
    sa.b = S.b;
    sa.phi = S.phi;
    sa.brick_flag = S.brick_flag;
    k_setup<<<ceil_div(g.ncell, 256), 256, 0, st>>>(sa);
    k_compact_bricks<<<1, 1024, 0, st>>>(S.brick_flag, S.nbricks, S.brick_list, S.d_nactive);
    ctx->launches += 2;
    FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(&ctx->h_misc[1], S.d_nactive, sizeof(int), cudaMemcpyDeviceToHost, st));

    PcgState h{};
    h.tol_mode = tol_mode;
    h.max_iters = max_iters;
    h.tol_abs = tol / scale;
    *S.st_host = h;
    FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(S.st, S.st_host, sizeof(PcgState), cudaMemcpyHostToDevice, st));

    PcgArgs A;
    A.B = B;
    A.list = S.brick_list;
    A.nactive = S.d_nactive;
    A.code = S.code;
    A.b = S.b;
    A.phi = S.phi;
    A.st = S.st;
    A.partials = S.partials;
    A.counter = S.counter;
    A.tol_abs = tol / scale;
    A.tol_rel = tol;
    A.skip_bb = rhs_override ? -1.0 : 1e-7 / (scale * scale);

    int rc;
    if (precision == FSIM_PREC_FP64) {
        if ((rc = alloc_fp64(ctx))) return rc;
        const size_t nc = (size_t)g.ncell;
        Vecs<double> v;
        v.r[0] = S.r64; v.r[1] = S.r64 + nc;
        v.s[0] = S.s64; v.s[1] = S.s64 + nc;
        v.z = S.z64; v.q = S.q64;
        v.x = S.phi;
        rc = run_pcg<double>(ctx, A, v, precision, stats);
    } else {
        const size_t nc = (size_t)g.ncell;
        Vecs<float> v;
        v.r[0] = S.r; v.r[1] = S.r + nc;
        v.s[0] = S.s; v.s[1] = S.s + nc;
        v.z = S.z; v.q = S.q;
        v.x = S.plo;
        rc = run_pcg<float>(ctx, A, v, precision, stats);
    }
    if (rc) return rc;
    PcgState& hs = *S.st_host;
    if (stats) {
        stats->residual_max = hs.rmax * scale;
        stats->residual_rel = hs.bb > 0 ? sqrt(hs.rr / hs.bb) : 0.0;
        stats->rhs_norm = sqrt(hs.bb) * scale;
        stats->num_active_bricks = ctx->h_misc[1];
    }
    if (hs.nan) {
        ctx->err = "pressure solve produced a non-finite scalar";
        return FSIM_E_NAN;
    }
    if (apply && !hs.skip) launch_apply_pressure(ctx, dt);
    return FSIM_OK;
}

namespace {
__global__ void k_rhs_out(GridGeom g, const double* b, const uint16_t* code, double scale, float* out) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)g.nx * g.ny * g.nz;
    if (j >= n) return;
    const long long c = (j / g.nz) * g.pz + (j % g.nz);
    out[j] = (code[c] & CODE_FLUID) ? (float)(b[c] * scale) : 0.f;
}
}  // namespace

// rhs of the last solve in the reference's units (b = scale * b')
void launch_rhs_out(fsim_ctx* ctx, float* out) {
    const GridGeom& g = ctx->g;
    const long long n = (long long)g.nx * g.ny * g.nz;
    k_rhs_out<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(g, ctx->sv.b, ctx->sv.code, ctx->sv.last_scale, out);
}
