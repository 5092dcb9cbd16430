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
#include "fsim_net.h"

#include <utility>

namespace {

// Programmatic dependent launch: the kernels of one PCG iteration are launched
// with programmatic stream serialisation, so each grid is scheduled while its
// predecessor drains.  Every such kernel lets its successor launch at once and
// then waits for its predecessor's completion (and memory) before touching any
// data, so the ordering of the stream is unchanged.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename... KArgs, typename... Args>
void launch_pdl(void (*kern)(KArgs...), unsigned grid, unsigned block, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

constexpr int BRX = 2, BRY = 4, BRZ = 32;
constexpr int PCG_THREADS = 256;
constexpr float TAU = 0.97f;
constexpr float SAFE = 0.25f;

// code bits
constexpr uint16_t CODE_FLUID = 0x8000;
// shared-memory copies of the codes (coarsest multigrid levels) also carry the
// cell's colour, (x + y + z) & 1, so that a half sweep needs no coordinates
constexpr uint16_t SCODE_ODD = 0x4000;
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

// cell t of active brick bb = {bx, by, bz, b} (the compacted list's coordinates)
__device__ __forceinline__ bool brick_cell(const BrickGeo& B, int4 bb, int t, int& x, int& y, int& z,
                                           long long& c) {
    x = bb.x * BRX + t / (BRY * BRZ);
    y = bb.y * BRY + (t / BRZ) % BRY;
    z = bb.z * BRZ + t % BRZ;
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
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    if (z >= g.nz) return;
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
// each entry holds the brick's coordinates and index, int4 {bx, by, bz, b}, so
// the kernels over active bricks take them with one load, not three divisions
__global__ void __launch_bounds__(1024) k_compact_bricks(const uint8_t* flag, long long nb, int nby, int nbz,
                                                         int4* xyz, int* count) {
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
        if (f) {
            const int pos = carry + before + __popc(bal & ((1u << lane) - 1u));
            const unsigned ju = (unsigned)j, t = ju / (unsigned)nbz, u = t / (unsigned)nby;
            xyz[pos] = make_int4((int)u, (int)(t - u * (unsigned)nby), (int)(ju - t * (unsigned)nbz), (int)j);
        }
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
    const int4* bxyz;  // active bricks, ascending: {bx, by, bz, b}
    const int* nactive;
    const uint16_t* code;
    const double* b;
    double* phi;
    PcgState* st;
    double* partials;
    unsigned* counter;
    double tol_abs, tol_rel;  // tolerance in A' units (abs) / relative
    double skip_bb;           // early-out threshold on b'.b' (reference: sum b^2 < 1e-7)
    int phi_zero;             // the solve starts from phi = 0 (its first residual is b)
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
    T rmaxT = (T)0;
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        const double* phi = a.phi;
        double ap = 0.0;
        if (!(first && a.phi_zero)) {  // from a zero start the first residual is b itself
            ap = (double)code_ns(cc) * phi[c];
#pragma unroll
            for (int k = 0; k < 6; k++)
                if ((cc >> k) & 1) ap -= phi[c + nb_off(a.B, k)];
        }
        const double bc = a.b[c];
        const double rv = bc - ap;
        const T rt = (T)rv;
        r[c] = rt;
        if (reset_x && sizeof(T) == 4) v.x[c] = (T)0;
        // FP64 runs at a small fraction of FP32 here: the max norms come from the
        // stored residual, and the rhs norms are needed by the first residual only
        acc[0] += rv * rv;
        rmaxT = fmax(rmaxT, fabs(rt));
        if (first) {
            acc[2] += bc * bc;
            acc[3] = fmax(acc[3], fabs(bc));
        }
    }
    acc[1] = fmax(acc[1], (double)rmaxT);
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
            const bool conv = (s->tol_mode == FSIM_TOL_ABS_MAX) ? (acc[1] < s->tol_abs) : (acc[0] <= s->tol_rel2);
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
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
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
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
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
    const bool beta0 = beta == 0.0;
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        // beta = 0 (first iteration, after a restart): s = z exactly, without
        // reading s_old (which may hold a previous solve's non-finite values)
        const T snc = beta0 ? v.z[c] : v.z[c] + betaT * so[c];
        T qv = (T)code_ns(cc) * snc;
#pragma unroll
        for (int k = 0; k < 6; k++)
            if ((cc >> k) & 1) {
                const long long j = c + nb_off(a.B, k);
                qv -= beta0 ? v.z[j] : v.z[j] + betaT * so[j];
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

// x += alpha s; r_new = r - alpha q; r.r, max|r|; then on r_new:
//   PMODE 1: the black half of the red-black IC solve (the red half is k_red)
//   PMODE 2: the first red-black Gauss-Seidel sweep of the multigrid V-cycle from
//            zero (red z = r/ns, black z = (r + sum_j r_j/ns_j)/ns)
template <typename T, int PMODE>
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
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        v.x[c] += alpha * s[c];
        const T rv = ro[c] - alpha * v.q[c];
        rn[c] = rv;
        rr.add(rv * rv);
        rmax = fmax(rmax, fabs(rv));
        if (PMODE != 0 && ((x + y + z) & 1)) {
            T sum = rv;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if ((cc >> k) & 1) {
                    const long long j = c + nb_off(a.B, k);
                    const uint16_t cj = a.code[j];
                    sum += (ro[j] - alpha * v.q[j]) * recip_ns<T>(code_ns(cj));
                }
            if (PMODE == 1) v.z[c] = sum * (T)black_pivot_inv(a.code, c, cc, a.B);
            else v.z[c] = sum * recip_ns<T>(code_ns(cc));
        } else if (PMODE == 2) {
            v.z[c] = rv * recip_ns<T>(code_ns(cc));
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
            const bool conv = (st->tol_mode == FSIM_TOL_ABS_MAX) ? (acc[1] < st->tol_abs) : (acc[0] <= st->tol_rel2);
            st->converged = conv ? 1 : 0;
            if (conv || st->it >= st->max_iters || !isfinite(acc[0])) st->done = 1;
            if (!isfinite(acc[0])) st->nan = 1;
            // the FP32 recursion is trusted for a fold_drop fall of r.r, then the
            // solution is folded into FP64 and the iteration restarts
            if (st->fold_enabled && acc[0] < st->fold_drop * st->rr_update) {
                st->need_fold = 1;
                st->done = 1;
            }
        }
    }
}

// ---- geometric multigrid preconditioner ------------------------------------
//
// z = M^-1 r by one V-cycle.  Level l + 1 halves every dimension (ceil); a
// coarse cell is fluid if any child is fluid, else air if any child is air,
// else solid.  Each level's operator is the same integer 7-point stencil
// rebuilt from its own cells (rediscretisation); in the fine level's units the
// level-l operator is L_l / 4^l, so the coarse right-hand side is
// 4 R (f - L x) with R the full-weighting restriction (R = P^T / 8, P the
// cell-centred trilinear prolongation, weights 3/4 and 1/4 per axis).  The
// smoother is red-black Gauss-Seidel, NU sweeps red->black before the coarse
// correction and black->red after it; the coarsest level (at most 4 cells per
// axis) is smoothed BOTTOM times each way inside one CTA.  Starting every level
// from zero, the V-cycle is a fixed symmetric linear operator, as CG requires.
// Sweeps per level group, first measured on the 256^3 fill workload (PCG to 1e-6,
// steps/s of the whole step; the defaults below were re-measured after the
// coarse levels got cheaper): (2, 2, 2) took 30 iterations; (3, 6, 6) 16.3
// iterations, 34.0 steps/s; (2, 6, 6) 17 iterations, 35.4; (1, 6, 6) 18.8, 35.8;
// (2, 4, 6) 17.8, 35.3.  A fine-level sweep costs ~107 us in place, a level-1
// sweep ~22 us: the coarse correction near the free surface is the weak part of
// the cycle, so coarse smoothing pays for itself and fine smoothing does not.
// MIXED precision: the FP32 recursion is folded into the FP64 solution (true
// FP64 residual, CG restart) each time the residual norm fell this many decades.
// The FP32 correction restarts from zero at every fold, so the drift between the
// recursive and the true residual stays near FP32 rounding of the fold's
// residual, far below a 10^-3 drop.  One decade per fold (the first setting)
// cost 5 refinements per 1e-6 solve at 256^3.
constexpr int MIXED_REFINE_DIGITS = 3;
// Per-level defaults re-measured on the 256^3 fill workload (steps/s, level 1 /
// deeper separate levels / cluster levels): 4/6/8 45.2, 4/8/6 45.0, 6/4/6 45.0,
// 5/5/8 44.9, 4/4/8 44.7 (18 iterations), 6/6/6 44.4, 4/8/10 44.0, 6/6/4 43.6.
// Level 0 with the free-surface band sweeps (steps/s on the same box; full
// sweeps / band sweeps): 2/0 46.8 (17.2 iterations), 1/0 47.8 (19.4), 1/2
// 48.7 (17.8), 1/3 49.3 (17.1), 1/4 49.0 (17.0), 1/5 48.6, 2/4 46.9 (16.0),
// 2/6 45.8: one full sweep plus three band sweeps recover the iterations a
// second full sweep saved, for about a third of its cost.  On smaller grids the
// band's launches cost more than the full sweep they replace (128^3 dam break:
// 173 -> 158 steps/s, 32^3: 480 -> 399), so the band is the default only from
// MG_BAND_MIN_CELLS cells on.
constexpr long long MG_BAND_MIN_CELLS = 1ll << 23;
constexpr int MG_NU_DEFAULT_BIG = 1;       // level 0, grids of MG_BAND_MIN_CELLS cells or more
constexpr int MG_NB_DEFAULT_BIG = 3;       // level 0 free-surface band, same grids
constexpr int MG_NU_DEFAULT = 2;           // level 0, smaller grids (no band)
constexpr int MG_NU_L1_DEFAULT = 4;        // level 1 (128^3 at 256^3)
constexpr int MG_NU_COARSE_DEFAULT = 6;    // deeper separately launched levels
constexpr int MG_NU_CLUSTER_DEFAULT = 8;   // cluster levels in global or distributed shared memory
constexpr int MG_NU_SMALL_DEFAULT = 6;     // levels rank 0 runs alone (<= 4096 cells): 8/6 45.5, 8/8 45.2,
                                           // 10/6 45.3, 12/4 45.3, 8/4 45.0 (17.75 iterations)
constexpr int MG_BOTTOM_SWEEPS = 4;  // on the <= 4^3 bottom level; 12 gave the same iterations, 12 us/it slower
constexpr int MG_BOTTOM_MAX = 4096;

struct MGLev {
    int nx, ny, nz, pz;
    const uint16_t* code;
    float* x;
    const float* f;
    const float* f1;  // level 0: the rhs is the current PCG residual buffer (r[0] or r[1])
    float* r;
};

__device__ __forceinline__ const float* mg_rhs(const PcgArgs& A, const MGLev& L) {
    return (L.f1 && (A.st->bufsel & 1)) ? L.f1 : L.f;
}

__device__ __forceinline__ long long mg_off(const MGLev& L, int k) {
    const long long st = (k >> 1) == 0 ? (long long)L.pz * L.ny : ((k >> 1) == 1 ? (long long)L.pz : 1ll);
    return (k & 1) ? -st : st;
}

// ---- quad kernels -----------------------------------------------------------
// Every multigrid kernel (and the MG-path PCG kernels) gives each thread a quad:
// four consecutive z cells of one row, 16-byte aligned (every level pads z to
// a multiple of 4).  The centre and the +-x / +-y neighbour quads are single
// float4 loads, the +-z neighbours come from the quad itself plus one scalar on
// either side, and the four cell codes are one 8-byte load.  Level 0 walks the
// active bricks (64 quads per 2x4x32 brick, four bricks per 256-thread pass);
// coarser levels walk all their quads.
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void unpack4(const float4 f, float (&v)[4]) {
    v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
}
__device__ __forceinline__ void codes4(const uint16_t* code, long long c0, uint16_t (&cc)[4]) {
    const uint2 w = *reinterpret_cast<const uint2*>(code + c0);
    cc[0] = (uint16_t)(w.x & 0xFFFFu);
    cc[1] = (uint16_t)(w.x >> 16);
    cc[2] = (uint16_t)(w.y & 0xFFFFu);
    cc[3] = (uint16_t)(w.y >> 16);
}
__device__ __forceinline__ bool any_fluid(const uint16_t (&cc)[4]) {
    return ((cc[0] | cc[1] | cc[2] | cc[3]) & CODE_FLUID) != 0;
}

// a field around a quad: centre and the four face-neighbour quads, plus z ends
struct Q7 {
    float c[4], xp[4], xm[4], yp[4], ym[4];
    float zm, zp;
};
// neighbour quads outside the level read as zero (their mask bits are clear)
__device__ __forceinline__ void load_q7(Q7& q, const float* v, long long c0, const MGLev& L, int x, int y, int z0) {
    const long long sx = (long long)L.pz * L.ny, sy = L.pz;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    unpack4(ld4(v + c0), q.c);
    unpack4(x + 1 < L.nx ? ld4(v + c0 + sx) : zero, q.xp);
    unpack4(x > 0 ? ld4(v + c0 - sx) : zero, q.xm);
    unpack4(y + 1 < L.ny ? ld4(v + c0 + sy) : zero, q.yp);
    unpack4(y > 0 ? ld4(v + c0 - sy) : zero, q.ym);
    q.zm = z0 > 0 ? v[c0 - 1] : 0.f;
    q.zp = z0 + 4 < L.pz ? v[c0 + 4] : 0.f;
}
__device__ __forceinline__ void codes4_nb(const uint16_t* code, long long c0, bool ok, uint16_t (&cc)[4]) {
    if (ok) codes4(code, c0, cc);
    else cc[0] = cc[1] = cc[2] = cc[3] = 0;
}
// sum over the fluid neighbours (mask bits of cc) of lane i
__device__ __forceinline__ float nbsum(const Q7& q, int i, uint16_t cc) {
    float s = 0.f;
    if (cc & 1) s += q.xp[i];
    if (cc & 2) s += q.xm[i];
    if (cc & 4) s += q.yp[i];
    if (cc & 8) s += q.ym[i];
    if (cc & 16) s += (i < 3) ? q.c[i + 1] : q.zp;
    if (cc & 32) s += (i > 0) ? q.c[i - 1] : q.zm;
    return s;
}

// all quads of a coarse level, thread i0 + k * step
// (x, y, z0) of quad i of a level, in 32-bit arithmetic (levels stay below 2^31 cells)
__device__ __forceinline__ void quad_xyz(const MGLev& L, long long i, int& x, int& y, int& z0) {
    const unsigned iu = (unsigned)i, qz = (unsigned)(L.pz >> 2), ny = (unsigned)L.ny;
    const unsigned t = iu / qz;
    z0 = (int)(iu - t * qz) << 2;
    const unsigned u = t / ny;
    y = (int)(t - u * ny);
    x = (int)u;
}

template <typename F>
__device__ __forceinline__ void mg_for_range(const MGLev& L, long long i0, long long step, F&& fn) {
    const long long n = (long long)L.nx * L.ny * (L.pz >> 2);
    for (long long i = i0; i < n; i += step) {
        int x, y, z0;
        quad_xyz(L, i, x, y, z0);
        fn(x, y, z0, ((long long)x * L.ny + y) * L.pz + z0);
    }
}

template <bool FINE, typename F>
__device__ __forceinline__ void mg_for_quads(const PcgArgs& A, const MGLev& L, F&& fn) {
    if (FINE) {
        const int nact = *A.nactive;
        const int sub = threadIdx.x >> 6, q = threadIdx.x & 63;
        for (int bk = blockIdx.x * 4 + sub; bk < nact; bk += gridDim.x * 4) {
            const int4 bb = A.bxyz[bk];
            const int x = bb.x * BRX + (q >> 5), y = bb.y * BRY + ((q >> 3) & 3), z0 = bb.z * BRZ + ((q & 7) << 2);
            if (x >= L.nx || y >= L.ny || z0 >= L.nz) continue;
            fn(x, y, z0, ((long long)x * L.ny + y) * L.pz + z0);
        }
    } else {
        mg_for_range(L, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, fn);
    }
}

__device__ __forceinline__ long long lev_sx(const MGLev& L) { return (long long)L.pz * L.ny; }

// one red-black Gauss-Seidel half sweep of a quad; first: the other colour is still zero
__device__ __forceinline__ void smooth_quad(const MGLev& L, const float* rhs, int color, int first, int x, int y,
                                            int z0, long long c0) {
    // every load is issued before the fluid test (one round trip, not two; the
    // levels sit in L2, so the loads of quads without fluid are cheap)
    uint16_t cc[4];
    codes4(L.code, c0, cc);
    float f[4];
    unpack4(ld4(rhs + c0), f);
    Q7 q;
    if (first) unpack4(ld4(L.x + c0), q.c);
    else load_q7(q, L.x, c0, L, x, y, z0);
    if (!any_fluid(cc)) return;
    const int par = (x + y + z0) & 1;
    float out[4] = {q.c[0], q.c[1], q.c[2], q.c[3]};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (((par ^ i) & 1) != color || !(cc[i] & CODE_FLUID)) continue;
        float sum = f[i];
        if (!first) sum += nbsum(q, i, cc[i]);
        out[i] = sum * c_rcp[code_ns(cc[i])];
    }
    st4(L.x + c0, out);
}

template <bool FINE>
__global__ void __launch_bounds__(PCG_THREADS) k_mg_smooth(const PcgArgs A, MGLev L, int color, int first) {
    pdl_enter();
    if (A.st->done) return;
    const float* rhs = mg_rhs(A, L);
    mg_for_quads<FINE>(A, L, [&](int x, int y, int z0, long long c0) { smooth_quad(L, rhs, color, first, x, y, z0, c0); });
}

// the last post-smoothing half sweep (red, level 0) fused with z.r (modes 0/1 as k_red)
__global__ void __launch_bounds__(PCG_THREADS) k_mg_smooth_dot(const PcgArgs A, MGLev L, int mode) {
    __shared__ double scratch[32];
    pdl_enter();
    if (A.st->done) return;
    const float* rhs = mg_rhs(A, L);
    Acc<float> zr;
    mg_for_quads<true>(A, L, [&](int x, int y, int z0, long long c0) {
        uint16_t cc[4];
        codes4(L.code, c0, cc);
        if (!any_fluid(cc)) return;
        float f[4];
        unpack4(ld4(rhs + c0), f);
        Q7 q;
        load_q7(q, L.x, c0, L, x, y, z0);
        const int par = (x + y + z0) & 1;
        float out[4] = {q.c[0], q.c[1], q.c[2], q.c[3]};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (!(cc[i] & CODE_FLUID)) continue;
            if (((par ^ i) & 1) == 0) out[i] = (f[i] + nbsum(q, i, cc[i])) * c_rcp[code_ns(cc[i])];
            zr.add(out[i] * f[i]);
        }
        st4(L.x + c0, out);
    });
    double acc[1] = {zr.value()};
    if (last_block_reduce<1>(acc, 0, A.partials, A.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* s = A.st;
            const double sig = acc[0];
            if (mode == 0) {
                s->beta = 0.0;
                s->sigma = sig;
                s->sigma_prev = sig;
            } else {
                s->beta = sig / s->sigma;
                s->sigma_prev = s->sigma;
                s->sigma = sig;
            }
            if (!isfinite(s->beta)) {
                s->nan = 1;
                s->done = 1;
            }
        }
    }
}

__device__ __forceinline__ void residual_quad(const MGLev& L, const float* rhs, int x, int y, int z0, long long c0) {
    uint16_t cc[4];
    codes4(L.code, c0, cc);
    float f[4];
    unpack4(ld4(rhs + c0), f);
    Q7 q;
    load_q7(q, L.x, c0, L, x, y, z0);
    if (!any_fluid(cc)) return;
    float out[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
        out[i] = (cc[i] & CODE_FLUID) ? f[i] - ((float)code_ns(cc[i]) * q.c[i] - nbsum(q, i, cc[i])) : 0.f;
    st4(L.r + c0, out);
}

template <bool FINE>
__global__ void __launch_bounds__(PCG_THREADS) k_mg_residual(const PcgArgs A, MGLev L) {
    pdl_enter();
    if (A.st->done) return;
    const float* rhs = mg_rhs(A, L);
    mg_for_quads<FINE>(A, L, [&](int x, int y, int z0, long long c0) { residual_quad(L, rhs, x, y, z0, c0); });
}

// coarse f = 0.5 * sum_fine P[f,C] r_f  (= 4 R r), per coarse quad:
// fine z 2 z0 - 1 .. 2 z0 + 8 come from the four fine quads at 2 z0 - 4 .. 2 z0 + 8
__device__ __forceinline__ void restrict_quad(const MGLev& F, const MGLev& Cl, int cx, int cy, int cz0, long long ci) {
    {
        uint16_t ccc[4];
        codes4(Cl.code, ci, ccc);
        if (!any_fluid(ccc)) return;
        float sum[4] = {0.f, 0.f, 0.f, 0.f};
        const int fz0 = 2 * cz0 - 4;  // first fine z loaded (a multiple of 4)
        for (int dx = -1; dx <= 2; dx++) {
            const int fx = 2 * cx + dx;
            if (fx < 0 || fx >= F.nx) continue;
            const float wx = (dx == 0 || dx == 1) ? 0.75f : 0.25f;
            for (int dy = -1; dy <= 2; dy++) {
                const int fy = 2 * cy + dy;
                if (fy < 0 || fy >= F.ny) continue;
                const float wxy = wx * ((dy == 0 || dy == 1) ? 0.75f : 0.25f);
                const long long row = ((long long)fx * F.ny + fy) * F.pz;
                // 16 fine values z = fz0 .. fz0 + 15, masked by fine fluid
                float fr[16];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int z = fz0 + 4 * k;
                    float v[4] = {0.f, 0.f, 0.f, 0.f};
                    if (z >= 0 && z < F.pz) {
                        // codes and residual loaded together; r is stale on quads
                        // without fluid (never written), so the codes mask it
                        uint16_t fc[4];
                        codes4(F.code, row + z, fc);
                        unpack4(ld4(F.r + row + z), v);
#pragma unroll
                        for (int e = 0; e < 4; e++)
                            if (!(fc[e] & CODE_FLUID)) v[e] = 0.f;
                    }
#pragma unroll
                    for (int e = 0; e < 4; e++) fr[4 * k + e] = v[e];
                }
                // coarse lane j takes fine 2(cz0+j) - 1 .. 2(cz0+j) + 2 = fr[3 + 2j .. 6 + 2j]
#pragma unroll
                for (int j = 0; j < 4; j++)
                    sum[j] += wxy * (0.25f * fr[3 + 2 * j] + 0.75f * fr[4 + 2 * j] + 0.75f * fr[5 + 2 * j] +
                                     0.25f * fr[6 + 2 * j]);
            }
        }
        float out[4];
        unpack4(ld4(Cl.f + ci), out);
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (ccc[j] & CODE_FLUID) out[j] = 0.5f * sum[j];
        st4(const_cast<float*>(Cl.f) + ci, out);
    }
}

__global__ void __launch_bounds__(PCG_THREADS) k_mg_restrict(const PcgState* st, MGLev F, MGLev Cl) {
    pdl_enter();
    if (st->done) return;
    mg_for_range(Cl, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x,
                 [&](int x, int y, int z0, long long c0) { restrict_quad(F, Cl, x, y, z0, c0); });
}

// fine x += P x_coarse on fluid fine cells, per fine quad: the quad's coarse z
// neighbours are z0/2 - 1 .. z0/2 + 2
__device__ __forceinline__ void prolong_quad(const MGLev& F, const MGLev& Cl, int x, int y, int z0, long long c0) {
    uint16_t cc[4];
    codes4(F.code, c0, cc);
    if (!any_fluid(cc)) return;
    const int px = (x & 1) ? x >> 1 : (x >> 1) - 1;  // lower coarse neighbour per axis
    const int py = (y & 1) ? y >> 1 : (y >> 1) - 1;
    const float wlx = (x & 1) ? 0.75f : 0.25f, wly = (y & 1) ? 0.75f : 0.25f;
    const int zc = (z0 >> 1) - 1;
    // coarse z zc .. zc + 3: with h = z0 / 2 even, either the quad at h plus the
    // value below it (h = 0 mod 4) or the quad at h - 2 plus the value above it
    const int hq = (z0 >> 1) & ~3;
    const bool lowq = ((z0 >> 1) & 3) == 0;
    const int ze = lowq ? zc : hq + 4;  // the extra value's z
    float sum[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int o = 0; o < 4; o++) {
        const int ox = o >> 1, oy = o & 1;
        const int cx = px + ox, cy = py + oy;
        if (cx < 0 || cy < 0 || cx >= Cl.nx || cy >= Cl.ny) continue;
        const float wxy = (ox ? 1.f - wlx : wlx) * (oy ? 1.f - wly : wly);
        const long long row = ((long long)cx * Cl.ny + cy) * Cl.pz;
        float qv[4];
        uint16_t qc[4];
        unpack4(ld4(Cl.x + row + hq), qv);
        codes4(Cl.code, row + hq, qc);
        const bool ein = ze >= 0 && ze < Cl.pz;
        const float ev = ein ? Cl.x[row + ze] : 0.f;
        const uint16_t ec = ein ? Cl.code[row + ze] : (uint16_t)0;
        float cv[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            // lowq: zc = hq - 1 (the extra value), then hq .. hq + 2; else hq + 1 .. hq + 3, then hq + 4
            const float v = lowq ? (k == 0 ? ev : qv[k - 1]) : (k == 3 ? ev : qv[k + 1]);
            const uint16_t c = lowq ? (k == 0 ? ec : qc[k - 1]) : (k == 3 ? ec : qc[k + 1]);
            cv[k] = (c & CODE_FLUID) ? v : 0.f;
        }
        // lanes: z0 (lower zc, w 1/4), z0+1 (zc+1, 3/4), z0+2 (zc+1, 1/4), z0+3 (zc+2, 3/4)
        sum[0] += wxy * (0.25f * cv[0] + 0.75f * cv[1]);
        sum[1] += wxy * (0.75f * cv[1] + 0.25f * cv[2]);
        sum[2] += wxy * (0.25f * cv[1] + 0.75f * cv[2]);
        sum[3] += wxy * (0.75f * cv[2] + 0.25f * cv[3]);
    }
    float xv[4];
    unpack4(ld4(F.x + c0), xv);
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (cc[i] & CODE_FLUID) xv[i] += sum[i];
    st4(F.x + c0, xv);
}

template <bool FINE>
__global__ void __launch_bounds__(PCG_THREADS) k_mg_prolong(const PcgArgs A, MGLev F, MGLev Cl) {
    pdl_enter();
    if (A.st->done) return;
    mg_for_quads<FINE>(A, F, [&](int x, int y, int z0, long long c0) { prolong_quad(F, Cl, x, y, z0, c0); });
}

// ---- free-surface band of the finest level ------------------------------------
// Quads with a fluid cell whose cells or six neighbouring cells include an
// interface cell (fluid with an air neighbour: fewer fluid than non-solid
// neighbours).  Extra red-black sweeps on this band only (mg_boundary_sweeps)
// target the error the coarse-grid correction leaves at the free surface,
// where the coarse levels represent the Dirichlet boundary worst.
__device__ __forceinline__ bool iface_cell(uint16_t c) { return (c & CODE_FLUID) && code_ns(c) != code_nf(c); }

__global__ void __launch_bounds__(PCG_THREADS) k_bnd_list(const PcgArgs A, MGLev L, int4* out, int* count) {
    const long long sx = lev_sx(L), sy = L.pz;
    mg_for_quads<true>(A, L, [&](int x, int y, int z0, long long c0) {
        uint16_t cc[4];
        codes4(L.code, c0, cc);
        if (!any_fluid(cc)) return;
        bool in = false;
        uint16_t nb[4];
#pragma unroll
        for (int i = 0; i < 4; i++) in |= iface_cell(cc[i]);
        codes4_nb(L.code, c0 + sx, x + 1 < L.nx, nb);
#pragma unroll
        for (int i = 0; i < 4; i++) in |= iface_cell(nb[i]);
        codes4_nb(L.code, c0 - sx, x > 0, nb);
#pragma unroll
        for (int i = 0; i < 4; i++) in |= iface_cell(nb[i]);
        codes4_nb(L.code, c0 + sy, y + 1 < L.ny, nb);
#pragma unroll
        for (int i = 0; i < 4; i++) in |= iface_cell(nb[i]);
        codes4_nb(L.code, c0 - sy, y > 0, nb);
#pragma unroll
        for (int i = 0; i < 4; i++) in |= iface_cell(nb[i]);
        if (z0 > 0) in |= iface_cell(L.code[c0 - 1]);
        if (z0 + 4 < L.pz) in |= iface_cell(L.code[c0 + 4]);
        if (in) out[atomicAdd(count, 1)] = make_int4(x, y, z0, 0);
    });
}

// one red-black half sweep over the band's quads
__global__ void __launch_bounds__(PCG_THREADS) k_mg_smooth_bnd(const PcgArgs A, MGLev L, const int4* list,
                                                               const int* count, int color) {
    pdl_enter();
    if (A.st->done) return;
    const float* rhs = mg_rhs(A, L);
    const int n = *count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 q = list[i];
        smooth_quad(L, rhs, color, 0, q.x, q.y, q.z, ((long long)q.x * L.ny + q.y) * L.pz + q.z);
    }
}

// ---- MG-path PCG kernels on quads (level 0, FP32) ------------------------------
// s_new = z + beta s_old; q = A' s_new; alpha = sigma / (s.q)
__global__ void __launch_bounds__(PCG_THREADS) k_spmv_q(const PcgArgs a, Vecs<float> v, MGLev L) {
    __shared__ double scratch[32];
    pdl_enter();
    if (a.st->done) return;
    const int sc = (a.st->bufsel >> 1) & 1;
    const float beta = (float)a.st->beta;
    const float* so = sc ? v.s[1] : v.s[0];
    float* sn = sc ? v.s[0] : v.s[1];
    Acc<float> sq;
    mg_for_quads<true>(a, L, [&](int x, int y, int z0, long long c0) {
        uint16_t cc[4];
        codes4(a.code, c0, cc);
        if (!any_fluid(cc)) return;
        Q7 zq;
        load_q7(zq, v.z, c0, L, x, y, z0);
        Q7 n = zq;  // s_new around the quad; beta = 0: s = z, s_old is not read
        if (beta != 0.f) {
            Q7 sq7;
            load_q7(sq7, so, c0, L, x, y, z0);
#pragma unroll
            for (int i = 0; i < 4; i++) {
                n.c[i] = zq.c[i] + beta * sq7.c[i];
                n.xp[i] = zq.xp[i] + beta * sq7.xp[i];
                n.xm[i] = zq.xm[i] + beta * sq7.xm[i];
                n.yp[i] = zq.yp[i] + beta * sq7.yp[i];
                n.ym[i] = zq.ym[i] + beta * sq7.ym[i];
            }
            n.zm = zq.zm + beta * sq7.zm;
            n.zp = zq.zp + beta * sq7.zp;
        }
        float qv[4], snc[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (cc[i] & CODE_FLUID) {
                snc[i] = n.c[i];
                qv[i] = (float)code_ns(cc[i]) * n.c[i] - nbsum(n, i, cc[i]);
                sq.add(snc[i] * qv[i]);
            } else {
                snc[i] = 0.f;
                qv[i] = 0.f;
            }
        }
        st4(sn + c0, snc);
        st4(v.q + c0, qv);
    });
    double acc[1] = {sq.value()};
    if (last_block_reduce<1>(acc, 0, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* s = a.st;
            s->alpha = s->sigma / acc[0];
            if (!isfinite(s->alpha)) {
                s->nan = 1;
                s->done = 1;
            }
            s->bufsel ^= 2;
        }
    }
}

// x += alpha s; r_new = r - alpha q; r.r, max|r|; first red-black sweep of the
// V-cycle from zero on r_new (red z = r/ns, black z = (r + sum_j r_j/ns_j)/ns)
__global__ void __launch_bounds__(PCG_THREADS) k_update_q(const PcgArgs a, Vecs<float> v, MGLev L) {
    __shared__ double scratch[32 * 2];
    pdl_enter();
    if (a.st->done) return;
    const int rc = a.st->bufsel & 1, sc = (a.st->bufsel >> 1) & 1;
    const float alpha = (float)a.st->alpha;
    const float* ro = rc ? v.r[1] : v.r[0];
    float* rn = rc ? v.r[0] : v.r[1];
    const float* s = sc ? v.s[1] : v.s[0];
    const long long sx = lev_sx(L), sy = L.pz;
    Acc<float> rr;
    float rmax = 0.f;
    mg_for_quads<true>(a, L, [&](int x, int y, int z0, long long c0) {
        uint16_t cc[4];
        codes4(a.code, c0, cc);
        if (!any_fluid(cc)) return;
        float sv[4], xv[4];
        unpack4(ld4(s + c0), sv);
        unpack4(ld4(v.x + c0), xv);
        Q7 rq, qq;
        load_q7(rq, ro, c0, L, x, y, z0);
        load_q7(qq, v.q, c0, L, x, y, z0);
        // neighbour codes for their 1/ns
        uint16_t cxp[4], cxm[4], cyp[4], cym[4];
        codes4_nb(a.code, c0 + sx, x + 1 < L.nx, cxp);
        codes4_nb(a.code, c0 - sx, x > 0, cxm);
        codes4_nb(a.code, c0 + sy, y + 1 < L.ny, cyp);
        codes4_nb(a.code, c0 - sy, y > 0, cym);
        const uint16_t czm = z0 > 0 ? a.code[c0 - 1] : 0, czp = z0 + 4 < L.pz ? a.code[c0 + 4] : 0;
        Q7 w;  // r_new / ns around the quad
        float rnc[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            rnc[i] = rq.c[i] - alpha * qq.c[i];
            w.c[i] = rnc[i] * c_rcp[code_ns(cc[i])];
            w.xp[i] = (rq.xp[i] - alpha * qq.xp[i]) * c_rcp[code_ns(cxp[i])];
            w.xm[i] = (rq.xm[i] - alpha * qq.xm[i]) * c_rcp[code_ns(cxm[i])];
            w.yp[i] = (rq.yp[i] - alpha * qq.yp[i]) * c_rcp[code_ns(cyp[i])];
            w.ym[i] = (rq.ym[i] - alpha * qq.ym[i]) * c_rcp[code_ns(cym[i])];
        }
        w.zm = (rq.zm - alpha * qq.zm) * c_rcp[code_ns(czm)];
        w.zp = (rq.zp - alpha * qq.zp) * c_rcp[code_ns(czp)];
        const int par = (x + y + z0) & 1;
        float zv[4], rout[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (!(cc[i] & CODE_FLUID)) {
                zv[i] = 0.f;
                rout[i] = 0.f;
                continue;
            }
            xv[i] += alpha * sv[i];
            rout[i] = rnc[i];
            rr.add(rnc[i] * rnc[i]);
            rmax = fmaxf(rmax, fabsf(rnc[i]));
            if (((par ^ i) & 1) == 0) zv[i] = w.c[i];  // red
            else zv[i] = (rnc[i] + nbsum(w, i, cc[i])) * c_rcp[code_ns(cc[i])];
        }
        st4(v.x + c0, xv);
        st4(rn + c0, rout);
        st4(v.z + c0, zv);
    });
    double acc[2] = {rr.value(), (double)rmax};
    if (last_block_reduce<2>(acc, 0x2, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) {
            PcgState* st = a.st;
            st->rr = acc[0];
            st->rmax = acc[1];
            st->it += 1;
            st->bufsel ^= 1;
            const bool conv = (st->tol_mode == FSIM_TOL_ABS_MAX) ? (acc[1] < st->tol_abs) : (acc[0] <= st->tol_rel2);
            st->converged = conv ? 1 : 0;
            if (conv || st->it >= st->max_iters || !isfinite(acc[0])) st->done = 1;
            if (!isfinite(acc[0])) st->nan = 1;
            if (st->fold_enabled && acc[0] < st->fold_drop * st->rr_update) {
                st->need_fold = 1;
                st->done = 1;
            }
        }
    }
}

// coarsest level: symmetric red-black Gauss-Seidel in shared memory, one CTA
__device__ void mg_bottom_block(const MGLev& L, float* sx, float* sf, uint16_t* sc) {
    const int n = L.nx * L.ny * L.nz;  // dense in shared memory, padded in global
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int z = i % L.nz, t = i / L.nz;
        const long long gi = (long long)t * L.pz + z;
        const int odd = (t / L.ny + t % L.ny + z) & 1;
        sx[i] = 0.f;
        sf[i] = L.f[gi];
        sc[i] = L.code[gi] | (odd ? SCODE_ODD : 0);
    }
    __syncthreads();
    const int sxs = L.ny * L.nz, sys = L.nz;
    for (int pass = 0; pass < 2 * MG_BOTTOM_SWEEPS; pass++) {
        // forward half: red then black; backward half: black then red
        for (int h = 0; h < 2; h++) {
            const int color = (pass < MG_BOTTOM_SWEEPS) ? h : 1 - h;
            const uint16_t want = CODE_FLUID | (color ? SCODE_ODD : 0);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const uint16_t cc = sc[i];
                if ((cc & (CODE_FLUID | SCODE_ODD)) != want) continue;
                float sum = sf[i];
                if (cc & 1) sum += sx[i + sxs];
                if (cc & 2) sum += sx[i - sxs];
                if (cc & 4) sum += sx[i + sys];
                if (cc & 8) sum += sx[i - sys];
                if (cc & 16) sum += sx[i + 1];
                if (cc & 32) sum += sx[i - 1];
                sx[i] = sum * c_rcp[code_ns(cc)];
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) L.x[(long long)(i / L.nz) * L.pz + (i % L.nz)] = sx[i];
}

__global__ void __launch_bounds__(1024) k_mg_bottom(const PcgState* st, MGLev L) {
    pdl_enter();
    if (st->done) return;
    __shared__ float sx[MG_BOTTOM_MAX];
    __shared__ float sf[MG_BOTTOM_MAX];
    __shared__ uint16_t sc[MG_BOTTOM_MAX];
    mg_bottom_block(L, sx, sf, sc);
}

// The coarse part of the V-cycle in one launch: levels lc .. last (lc's rhs was
// restricted by the caller) run by one thread-block cluster, the passes over a
// level separated by cluster barriers (release/acquire at cluster scope, so
// each pass sees the previous pass's global writes).  Replaces ~11 launches per
// level of latency-bound small kernels.
constexpr int MG_MAX_LEVELS = 12;
constexpr int MG_CLUSTER_THREADS = 1024;
// Largest level handed to the cluster kernel.  At 256^3 the 64^3 level (262k
// cells) ran ~8 us per pass on the cluster's 16 SMs and is faster as separate
// full-GPU launches (35.6 -> 37.5 steps/s); moving the 32^3 level out as well
// changed nothing.
constexpr long long MG_CLUSTER_CELLS = 40000;
constexpr int MG_CLUSTER_SMEM = 200 * 1024;  // dynamic shared memory limit of the cluster kernel

struct MGChain {
    MGLev lev[MG_MAX_LEVELS];
    int lc, last, nu;
    int nu_small;  // sweeps on the shared-memory levels ls .. last-1
    int ls;  // first level small enough to run in one CTA's shared memory (<= last)
    // levels lc .. ls-1 as x slabs in distributed shared memory (slab != 0):
    // planes per CTA and float offset of each level in the pool, then the offset
    // of rank 0's shared-memory levels
    int slab;
    int P[MG_MAX_LEVELS];
    int off[MG_MAX_LEVELS];
    int soff;
};

// ---- the smallest levels in one CTA's shared memory ----------------------------
// Levels with at most MG_SMEM_CELLS cells are copied (dense, z fastest) into
// shared memory and run their part of the V-cycle there: the same red-black
// Gauss-Seidel, full-weighting restriction (x 0.5) and trilinear prolongation
// as the global kernels, with __syncthreads between passes instead of cluster
// barriers and global-memory round trips.
constexpr int MG_SMEM_CELLS = 4096;

struct SLev {
    int nx, ny, nz, n;
    float *x, *f, *r;
    uint16_t* code;
};

__device__ __forceinline__ int sidx(const SLev& L, int x, int y, int z) { return (x * L.ny + y) * L.nz + z; }

// Each thread holds at most four cells of a shared-memory level (<= 4096 cells,
// 1024 threads): a pass computes all of them before it stores any, so their
// loads overlap (a half sweep's cells read only the other colour)
constexpr int SCELLS_PER_THREAD = 4;
static_assert(SCELLS_PER_THREAD * MG_CLUSTER_THREADS >= MG_SMEM_CELLS, "shared-memory level cells per thread");

__device__ __forceinline__ float s_nbsum(const SLev& L, int i, uint16_t cc, int sx, int sy) {
    float s = 0.f;
    if (cc & 1) s += L.x[i + sx];
    if (cc & 2) s += L.x[i - sx];
    if (cc & 4) s += L.x[i + sy];
    if (cc & 8) s += L.x[i - sy];
    if (cc & 16) s += L.x[i + 1];
    if (cc & 32) s += L.x[i - 1];
    return s;
}

__device__ void s_smooth(const SLev L, int color) {
    const int sx = L.ny * L.nz, sy = L.nz;
    const uint16_t want = CODE_FLUID | (color ? SCODE_ODD : 0);
    float nv[SCELLS_PER_THREAD];
    bool act[SCELLS_PER_THREAD];
#pragma unroll
    for (int k = 0; k < SCELLS_PER_THREAD; k++) {
        const int i = threadIdx.x + k * MG_CLUSTER_THREADS;
        act[k] = false;
        nv[k] = 0.f;
        if (i >= L.n) continue;
        const uint16_t cc = L.code[i];
        if ((cc & (CODE_FLUID | SCODE_ODD)) != want) continue;
        act[k] = true;
        nv[k] = (L.f[i] + s_nbsum(L, i, cc, sx, sy)) * c_rcp[code_ns(cc)];
    }
#pragma unroll
    for (int k = 0; k < SCELLS_PER_THREAD; k++)
        if (act[k]) L.x[threadIdx.x + k * MG_CLUSTER_THREADS] = nv[k];
    __syncthreads();
}

__device__ void s_residual(const SLev L) {
    const int sx = L.ny * L.nz, sy = L.nz;
    float rv[SCELLS_PER_THREAD];
#pragma unroll
    for (int k = 0; k < SCELLS_PER_THREAD; k++) {
        const int i = threadIdx.x + k * MG_CLUSTER_THREADS;
        rv[k] = 0.f;
        if (i >= L.n) continue;
        const uint16_t cc = L.code[i];
        if (cc & CODE_FLUID) rv[k] = L.f[i] - ((float)code_ns(cc) * L.x[i] - s_nbsum(L, i, cc, sx, sy));
    }
#pragma unroll
    for (int k = 0; k < SCELLS_PER_THREAD; k++) {
        const int i = threadIdx.x + k * MG_CLUSTER_THREADS;
        if (i < L.n) L.r[i] = rv[k];
    }
    __syncthreads();
}

__device__ __forceinline__ float fw_weight(int d) { return (d == 0 || d == 1) ? 0.75f : 0.25f; }

// coarse f = 0.5 * sum_fine P r (fine fluid only), coarse x = 0
__device__ void s_restrict(const SLev F, const SLev C) {
    for (int i = threadIdx.x; i < C.n; i += blockDim.x) {
        const int cz = i % C.nz, cy = (i / C.nz) % C.ny, cx = i / (C.nz * C.ny);
        C.x[i] = 0.f;
        if (!(C.code[i] & CODE_FLUID)) {
            C.f[i] = 0.f;
            continue;
        }
        // the fine residual is zero off the fine fluid cells (s_residual)
        float sum = 0.f;
#pragma unroll
        for (int dx = -1; dx <= 2; dx++) {
            const int fx = 2 * cx + dx;
            if (fx < 0 || fx >= F.nx) continue;
#pragma unroll
            for (int dy = -1; dy <= 2; dy++) {
                const int fy = 2 * cy + dy;
                if (fy < 0 || fy >= F.ny) continue;
                const float wxy = fw_weight(dx) * fw_weight(dy);
                const int row = sidx(F, fx, fy, 0);
#pragma unroll
                for (int dz = -1; dz <= 2; dz++) {
                    const int fz = 2 * cz + dz;
                    if (fz < 0 || fz >= F.nz) continue;
                    sum += wxy * fw_weight(dz) * F.r[row + fz];
                }
            }
        }
        C.f[i] = 0.5f * sum;
    }
    __syncthreads();
}

// fine x += P x_coarse on fluid fine cells (coarse fluid values only)
__device__ void s_prolong(const SLev F, const SLev C) {
    for (int i = threadIdx.x; i < F.n; i += blockDim.x) {
        if (!(F.code[i] & CODE_FLUID)) continue;
        const int z = i % F.nz, y = (i / F.nz) % F.ny, x = i / (F.nz * F.ny);
        const int p[3] = {(x & 1) ? x >> 1 : (x >> 1) - 1, (y & 1) ? y >> 1 : (y >> 1) - 1,
                          (z & 1) ? z >> 1 : (z >> 1) - 1};
        const float wl[3] = {(x & 1) ? 0.75f : 0.25f, (y & 1) ? 0.75f : 0.25f, (z & 1) ? 0.75f : 0.25f};
        float sum = 0.f;
        for (int o = 0; o < 8; o++) {
            const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
            const int cx = p[0] + ox, cy = p[1] + oy, cz = p[2] + oz;
            if (cx < 0 || cy < 0 || cz < 0 || cx >= C.nx || cy >= C.ny || cz >= C.nz) continue;
            const int ci = sidx(C, cx, cy, cz);
            if (!(C.code[ci] & CODE_FLUID)) continue;
            sum += (ox ? 1.f - wl[0] : wl[0]) * (oy ? 1.f - wl[1] : wl[1]) * (oz ? 1.f - wl[2] : wl[2]) * C.x[ci];
        }
        F.x[i] += sum;
    }
    __syncthreads();
}

// Levels ls..last in one CTA's shared memory, dense (z fastest), laid out from
// `smem` level by level: x, f, r (n floats each), then the codes (n uint16,
// padded to whole floats).  load_f: level ls's rhs comes from global memory
// (otherwise the caller's restriction writes it into this layout).
__device__ void smem_levels_init(const MGChain& C, float* smem, SLev* S, bool load_f) {
    if (threadIdx.x == 0) {
        float* p = smem;
        for (int l = C.ls; l <= C.last; l++) {
            const MGLev& G = C.lev[l];
            SLev& L = S[l];
            L.nx = G.nx; L.ny = G.ny; L.nz = G.nz;
            L.n = G.nx * G.ny * G.nz;
            L.x = p; p += L.n;
            L.f = p; p += L.n;
            L.r = p; p += L.n;
            L.code = reinterpret_cast<uint16_t*>(p);
            p += (L.n + 1) / 2;
        }
    }
    __syncthreads();
    for (int l = C.ls; l <= C.last; l++) {
        const MGLev& G = C.lev[l];
        const SLev L = S[l];
        for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
            const int z = i % L.nz, t = i / L.nz;
            const long long gi = (long long)t * G.pz + z;
            const int odd = (t / L.ny + t % L.ny + z) & 1;
            L.code[i] = G.code[gi] | (odd ? SCODE_ODD : 0);
            L.x[i] = 0.f;
            if (l == C.ls && load_f) L.f[i] = G.f[gi];
        }
    }
    __syncthreads();
}

// the V-cycle over those levels; store_x: level ls's correction goes back to
// global memory (otherwise the caller's prolongation reads it in place)
__device__ void smem_levels_run(const MGChain& C, const SLev* S, bool store_x) {
    for (int l = C.ls; l < C.last; l++) {
        for (int k = 0; k < C.nu_small; k++) {
            s_smooth(S[l], 0);
            s_smooth(S[l], 1);
        }
        s_residual(S[l]);
        s_restrict(S[l], S[l + 1]);
    }
    for (int k = 0; k < MG_BOTTOM_SWEEPS; k++) {
        s_smooth(S[C.last], 0);
        s_smooth(S[C.last], 1);
    }
    for (int k = 0; k < MG_BOTTOM_SWEEPS; k++) {
        s_smooth(S[C.last], 1);
        s_smooth(S[C.last], 0);
    }
    for (int l = C.last - 1; l >= C.ls; l--) {
        s_prolong(S[l], S[l + 1]);
        for (int k = 0; k < C.nu_small; k++) {
            s_smooth(S[l], 1);
            s_smooth(S[l], 0);
        }
    }
    if (store_x) {
        const MGLev& G = C.lev[C.ls];
        for (int i = threadIdx.x; i < S[C.ls].n; i += blockDim.x)
            G.x[(long long)(i / S[C.ls].nz) * G.pz + (i % S[C.ls].nz)] = S[C.ls].x[i];
    }
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned n;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
    return n;
}


// ---- cluster levels held in distributed shared memory ------------------------
// With MGChain::slab set, every CTA of the cluster holds P consecutive x planes
// of each level lc .. ls-1 in its own shared memory (x, f, r and the codes, at
// the same offsets in every CTA) and reads its neighbours' boundary planes
// through distributed shared memory; the cluster barrier separates the passes.
// The restriction into level ls writes straight into rank 0's shared-memory
// levels, and the prolongation from ls reads them there, so only level lc's
// rhs comes from global memory and only its correction goes back.
constexpr uint16_t SCODE_XLO = 0x2000;  // slab copies: x - 1 lies in the previous CTA
constexpr uint16_t SCODE_XHI = 0x1000;  // slab copies: x + 1 lies in the next CTA

struct DLev {
    float *x, *f, *r;
    uint16_t* code;
    int nx, ny, nz, P, np, x0, plane;
};

__device__ __forceinline__ DLev dlev(const MGChain& C, int l, float* pool, unsigned rank) {
    const MGLev& G = C.lev[l];
    DLev D;
    D.nx = G.nx; D.ny = G.ny; D.nz = G.nz;
    D.P = C.P[l];
    D.plane = G.ny * G.nz;
    D.x0 = (int)rank * D.P;
    D.np = max(0, min(D.P, G.nx - D.x0));
    const int m = D.P * D.plane;
    float* p = pool + C.off[l];
    D.x = p;
    D.f = p + m;
    D.r = p + 2 * m;
    D.code = reinterpret_cast<uint16_t*>(p + 3 * m);
    return D;
}

// the same shared-memory location in cluster CTA `rank` (generic address)
template <typename T>
__device__ __forceinline__ T* dsm(T* p, unsigned rank) {
    unsigned long long out;
    asm("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(reinterpret_cast<unsigned long long>(p)), "r"(rank));
    return reinterpret_cast<T*>(out);
}

__device__ __forceinline__ float slab_nbsum(const DLev& D, int i, uint16_t cc, const float* xp, const float* xn) {
    float s = 0.f;
    if (cc & 1) s += (cc & SCODE_XHI) ? xn[i - (D.np - 1) * D.plane] : D.x[i + D.plane];
    if (cc & 2) s += (cc & SCODE_XLO) ? xp[i + (D.P - 1) * D.plane] : D.x[i - D.plane];
    if (cc & 4) s += D.x[i + D.nz];
    if (cc & 8) s += D.x[i - D.nz];
    if (cc & 16) s += D.x[i + 1];
    if (cc & 32) s += D.x[i - 1];
    return s;
}

// red-black half sweep; first: the other colour is still zero
__device__ void slab_smooth(const DLev& D, int color, bool first, const float* xp, const float* xn) {
    const uint16_t want = CODE_FLUID | (color ? SCODE_ODD : 0);
    const int n = D.np * D.plane;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint16_t cc = D.code[i];
        if ((cc & (CODE_FLUID | SCODE_ODD)) != want) continue;
        float sum = D.f[i];
        if (!first) sum += slab_nbsum(D, i, cc, xp, xn);
        D.x[i] = sum * c_rcp[code_ns(cc)];
    }
}

__device__ void slab_residual(const DLev& D, const float* xp, const float* xn) {
    const int n = D.np * D.plane;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint16_t cc = D.code[i];
        float rv = 0.f;
        if (cc & CODE_FLUID) rv = D.f[i] - ((float)code_ns(cc) * D.x[i] - slab_nbsum(D, i, cc, xp, xn));
        D.r[i] = rv;
    }
}

// coarse f = 0.5 * sum_fine P r from level l's slabs (r is zero off the fluid)
// into level l + 1: the CTA's own slab, or rank 0's first shared-memory level
// (its cells spread over the whole cluster)
__device__ void slab_restrict(const MGChain& C, int l, float* pool, unsigned rank, unsigned cs, float* spool) {
    const DLev F = dlev(C, l, pool, rank);
    const MGLev& Gc = C.lev[l + 1];
    const bool to_slab = l + 1 < C.ls;
    const DLev D = dlev(C, l + 1, pool, rank);  // used only when to_slab
    const int nsm = Gc.nx * Gc.ny * Gc.nz;
    const int n = to_slab ? D.np * D.plane : nsm;
    const int i0 = to_slab ? (int)threadIdx.x : (int)(rank * blockDim.x + threadIdx.x);
    const int step = to_slab ? (int)blockDim.x : (int)(cs * blockDim.x);
    float* fout = to_slab ? D.f : dsm(spool + nsm, 0);
    const uint16_t* cin = to_slab ? D.code : reinterpret_cast<const uint16_t*>(dsm(spool + 3 * nsm, 0));
    for (int i = i0; i < n; i += step) {
        int cx, cy, cz;
        if (to_slab) {
            const int xl = i / D.plane, t = i - xl * D.plane;
            cx = D.x0 + xl;
            cy = t / Gc.nz;
            cz = t - cy * Gc.nz;
        } else {
            cz = i % Gc.nz;
            const int t = i / Gc.nz;
            cy = t % Gc.ny;
            cx = t / Gc.ny;
        }
        if (!(cin[i] & CODE_FLUID)) {
            fout[i] = 0.f;
            continue;
        }
        float sum = 0.f;
        for (int dx = -1; dx <= 2; dx++) {
            const int fx = 2 * cx + dx;
            if (fx < 0 || fx >= F.nx) continue;
            const unsigned ro = (unsigned)(fx / F.P);
            const float* rp = (ro == rank ? F.r : dsm(F.r, ro)) + (fx - (int)ro * F.P) * F.plane;
#pragma unroll
            for (int dy = -1; dy <= 2; dy++) {
                const int fy = 2 * cy + dy;
                if (fy < 0 || fy >= F.ny) continue;
                const float wxy = fw_weight(dx) * fw_weight(dy);
                const float* row = rp + fy * F.nz;
#pragma unroll
                for (int dz = -1; dz <= 2; dz++) {
                    const int fz = 2 * cz + dz;
                    if (fz < 0 || fz >= F.nz) continue;
                    sum += wxy * fw_weight(dz) * row[fz];
                }
            }
        }
        fout[i] = 0.5f * sum;
    }
}

// fine x += P x_coarse on level l's fluid cells (coarse fluid values only), the
// coarse level being level l + 1's slabs or rank 0's first shared-memory level
__device__ void slab_prolong(const MGChain& C, int l, float* pool, unsigned rank, float* spool) {
    const DLev F = dlev(C, l, pool, rank);
    const MGLev& Gc = C.lev[l + 1];
    const bool from_slab = l + 1 < C.ls;
    const DLev D = dlev(C, l + 1, pool, rank);  // used only when from_slab
    const int nsm = Gc.nx * Gc.ny * Gc.nz;
    const float* sx0 = from_slab ? nullptr : dsm(spool, 0);
    const uint16_t* sc0 = from_slab ? nullptr : reinterpret_cast<const uint16_t*>(dsm(spool + 3 * nsm, 0));
    const int n = F.np * F.plane;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (!(F.code[i] & CODE_FLUID)) continue;
        const int xl = i / F.plane, t = i - xl * F.plane;
        const int x = F.x0 + xl, y = t / F.nz, z = t - y * F.nz;
        const int p[3] = {(x & 1) ? x >> 1 : (x >> 1) - 1, (y & 1) ? y >> 1 : (y >> 1) - 1,
                          (z & 1) ? z >> 1 : (z >> 1) - 1};
        const float wl[3] = {(x & 1) ? 0.75f : 0.25f, (y & 1) ? 0.75f : 0.25f, (z & 1) ? 0.75f : 0.25f};
        float sum = 0.f;
#pragma unroll
        for (int o = 0; o < 8; o++) {
            const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
            const int cx = p[0] + ox, cy = p[1] + oy, cz = p[2] + oz;
            if (cx < 0 || cy < 0 || cz < 0 || cx >= Gc.nx || cy >= Gc.ny || cz >= Gc.nz) continue;
            float v;
            uint16_t c;
            if (from_slab) {
                const unsigned ro = (unsigned)(cx / D.P);
                const int li = ((cx - (int)ro * D.P) * Gc.ny + cy) * Gc.nz + cz;
                v = (ro == rank ? D.x : dsm(D.x, ro))[li];
                c = (ro == rank ? D.code : dsm(D.code, ro))[li];
            } else {
                const int ci = (cx * Gc.ny + cy) * Gc.nz + cz;
                v = sx0[ci];
                c = sc0[ci];
            }
            if (!(c & CODE_FLUID)) continue;
            sum += (ox ? 1.f - wl[0] : wl[0]) * (oy ? 1.f - wl[1] : wl[1]) * (oz ? 1.f - wl[2] : wl[2]) * v;
        }
        F.x[i] += sum;
    }
}

__global__ void __launch_bounds__(MG_CLUSTER_THREADS) k_mg_coarse(const PcgArgs A, const __grid_constant__ MGChain C) {
    pdl_enter();
    if (A.st->done) return;  // the same value in every CTA of the cluster
    extern __shared__ float pool[];
    __shared__ SLev S[MG_MAX_LEVELS];
    const unsigned rank = cluster_rank(), cs = cluster_size();
    if (C.slab) {
        float* spool = pool + C.soff;
        for (int l = C.lc; l < C.ls; l++) {
            const DLev D = dlev(C, l, pool, rank);
            const MGLev& G = C.lev[l];
            for (int i = threadIdx.x; i < D.np * D.plane; i += blockDim.x) {
                const int xl = i / D.plane, t = i - xl * D.plane, y = t / D.nz, z = t - y * D.nz;
                const long long gi = ((long long)(D.x0 + xl) * G.ny + y) * G.pz + z;
                uint16_t cc = G.code[gi];
                if ((D.x0 + xl + y + z) & 1) cc |= SCODE_ODD;
                if (xl == 0) cc |= SCODE_XLO;
                if (xl == D.np - 1) cc |= SCODE_XHI;
                D.code[i] = cc;
                D.x[i] = 0.f;
                if (l == C.lc) D.f[i] = G.f[gi];
            }
        }
        if (rank == 0) smem_levels_init(C, spool, S, false);
        cluster_barrier();
        for (int l = C.lc; l < C.ls; l++) {
            const DLev D = dlev(C, l, pool, rank);
            const float* xp = rank > 0 ? dsm(D.x, rank - 1) : nullptr;
            const float* xn = rank + 1 < cs ? dsm(D.x, rank + 1) : nullptr;
            for (int k = 0; k < C.nu; k++) {
                slab_smooth(D, 0, k == 0, xp, xn);
                cluster_barrier();
                slab_smooth(D, 1, false, xp, xn);
                cluster_barrier();
            }
            slab_residual(D, xp, xn);
            cluster_barrier();
            slab_restrict(C, l, pool, rank, cs, spool);
            cluster_barrier();
        }
        if (rank == 0) smem_levels_run(C, S, false);
        cluster_barrier();
        for (int l = C.ls - 1; l >= C.lc; l--) {
            const DLev D = dlev(C, l, pool, rank);
            const float* xp = rank > 0 ? dsm(D.x, rank - 1) : nullptr;
            const float* xn = rank + 1 < cs ? dsm(D.x, rank + 1) : nullptr;
            slab_prolong(C, l, pool, rank, spool);
            cluster_barrier();
            for (int k = 0; k < C.nu; k++) {
                slab_smooth(D, 1, false, xp, xn);
                cluster_barrier();
                slab_smooth(D, 0, false, xp, xn);
                cluster_barrier();
            }
        }
        // level lc's correction back to global memory (its slab alone: no other
        // CTA reads this CTA's shared memory after the last barrier)
        const DLev D = dlev(C, C.lc, pool, rank);
        const MGLev& G = C.lev[C.lc];
        for (int i = threadIdx.x; i < D.np * D.plane; i += blockDim.x) {
            const int xl = i / D.plane, t = i - xl * D.plane, y = t / D.nz, z = t - y * D.nz;
            G.x[((long long)(D.x0 + xl) * G.ny + y) * G.pz + z] = D.x[i];
        }
        return;
    }
    const long long i0 = (long long)rank * blockDim.x + threadIdx.x;
    const long long step = (long long)cs * blockDim.x;
    for (int l = C.lc; l < C.ls; l++) {
        const MGLev& L = C.lev[l];
        for (int k = 0; k < C.nu; k++) {
            mg_for_range(L, i0, step, [&](int x, int y, int z0, long long c0) { smooth_quad(L, L.f, 0, k == 0, x, y, z0, c0); });
            cluster_barrier();
            mg_for_range(L, i0, step, [&](int x, int y, int z0, long long c0) { smooth_quad(L, L.f, 1, 0, x, y, z0, c0); });
            cluster_barrier();
        }
        mg_for_range(L, i0, step, [&](int x, int y, int z0, long long c0) { residual_quad(L, L.f, x, y, z0, c0); });
        cluster_barrier();
        const MGLev& Cl = C.lev[l + 1];
        mg_for_range(Cl, i0, step, [&](int x, int y, int z0, long long c0) { restrict_quad(L, Cl, x, y, z0, c0); });
        cluster_barrier();
    }
    if (rank == 0) {
        smem_levels_init(C, pool, S, true);
        smem_levels_run(C, S, true);
    }
    cluster_barrier();
    for (int l = C.ls - 1; l >= C.lc; l--) {
        const MGLev& L = C.lev[l];
        const MGLev& Cl = C.lev[l + 1];
        mg_for_range(L, i0, step, [&](int x, int y, int z0, long long c0) { prolong_quad(L, Cl, x, y, z0, c0); });
        cluster_barrier();
        for (int k = 0; k < C.nu; k++) {
            mg_for_range(L, i0, step, [&](int x, int y, int z0, long long c0) { smooth_quad(L, L.f, 1, 0, x, y, z0, c0); });
            cluster_barrier();
            mg_for_range(L, i0, step, [&](int x, int y, int z0, long long c0) { smooth_quad(L, L.f, 0, 0, x, y, z0, c0); });
            cluster_barrier();
        }
    }
}

// coarse cell kinds: fluid if any child is fluid, else air if any child is air
__global__ void k_mg_coarsen(MGLev F, const uint8_t* fkind, const uint8_t* fflags, MGLev Cl, uint8_t* ckind) {
    const long long n = (long long)Cl.nx * Cl.ny * Cl.nz;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned iu = (unsigned)i, t = iu / (unsigned)Cl.nz, u = t / (unsigned)Cl.ny;
    const int cz = (int)(iu - t * (unsigned)Cl.nz), cy = (int)(t - u * (unsigned)Cl.ny), cx = (int)u;
    const long long ci = ((long long)cx * Cl.ny + cy) * Cl.pz + cz;
    int best = 2;
    for (int o = 0; o < 8; o++) {
        const int fx = 2 * cx + (o >> 2), fy = 2 * cy + ((o >> 1) & 1), fz = 2 * cz + (o & 1);
        if (fx >= F.nx || fy >= F.ny || fz >= F.nz) continue;
        const long long fi = ((long long)fx * F.ny + fy) * F.pz + fz;
        int k;
        if (fkind) k = fkind[fi];
        else k = (F.code[fi] & CODE_FLUID) ? 0 : (fflags[fi] == C_AIR ? 1 : 2);
        best = min(best, k);
    }
    ckind[ci] = (uint8_t)best;
}

// per-cell code of a coarse level from its kinds (outside the level = solid)
__global__ void k_mg_code(MGLev L, const uint8_t* kind, uint16_t* code) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned iu = (unsigned)i, t = iu / (unsigned)L.nz, u = t / (unsigned)L.ny;
    const int z = (int)(iu - t * (unsigned)L.nz), y = (int)(t - u * (unsigned)L.ny), x = (int)u;
    const long long ci = ((long long)x * L.ny + y) * L.pz + z;
    if (kind[ci] != 0) {
        code[ci] = 0;
        return;
    }
    uint16_t cd = CODE_FLUID;
    int ns = 0;
    const int pos[3] = {x, y, z}, lim[3] = {L.nx, L.ny, L.nz};
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const int a = k >> 1, dir = (k & 1) ? -1 : 1;
        const int q = pos[a] + dir;
        if (q < 0 || q >= lim[a]) continue;
        const uint8_t kn = kind[ci + mg_off(L, k)];
        if (kn == 0) cd |= (uint16_t)(1u << k);
        if (kn != 2) ns++;
    }
    code[ci] = cd | (uint16_t)(ns << 8);
}

// phi += x; x = 0   (fold the FP32 accumulator into the FP64 solution)
__global__ void __launch_bounds__(PCG_THREADS) k_fold(const PcgArgs a, float* x) {
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int xx, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, xx, y, z, c)) continue;
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
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.brick_xyz, S.nbricks * sizeof(int4)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.d_nactive, sizeof(int)));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.brick_flag, S.nbricks));
    FSIM_CUDA_TRY(ctx, cudaMalloc(&S.code, nc * sizeof(uint16_t)));
    FSIM_CUDA_TRY(ctx, cudaMemset(S.code, 0, nc * sizeof(uint16_t)));
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_update<float, 1>, PCG_THREADS, 0);
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
    // multigrid hierarchy: halve until every dimension is <= 4
    MGLevelBufs l0;
    l0.nx = g.nx; l0.ny = g.ny; l0.nz = g.nz; l0.pz = g.pz; l0.ncell = g.ncell;
    l0.code = S.code;
    FSIM_CUDA_TRY(ctx, cudaMalloc(&l0.r, nc * sizeof(float)));
    FSIM_CUDA_TRY(ctx, cudaMemset(l0.r, 0, nc * sizeof(float)));
    S.mg.push_back(l0);
    while (std::max(S.mg.back().nx, std::max(S.mg.back().ny, S.mg.back().nz)) > 4) {
        const MGLevelBufs& f = S.mg.back();
        MGLevelBufs c;
        c.nx = (f.nx + 1) / 2; c.ny = (f.ny + 1) / 2; c.nz = (f.nz + 1) / 2; c.pz = (c.nz + 3) & ~3;
        c.ncell = (long long)c.nx * c.ny * c.pz;
        FSIM_CUDA_TRY(ctx, cudaMalloc(&c.kind, c.ncell));
        FSIM_CUDA_TRY(ctx, cudaMalloc(&c.code, c.ncell * sizeof(uint16_t)));
        FSIM_CUDA_TRY(ctx, cudaMalloc(&c.x, c.ncell * sizeof(float)));
        FSIM_CUDA_TRY(ctx, cudaMalloc(&c.f, c.ncell * sizeof(float)));
        FSIM_CUDA_TRY(ctx, cudaMalloc(&c.r, c.ncell * sizeof(float)));
        FSIM_CUDA_TRY(ctx, cudaMemset(c.x, 0, c.ncell * sizeof(float)));
        FSIM_CUDA_TRY(ctx, cudaMemset(c.f, 0, c.ncell * sizeof(float)));
        FSIM_CUDA_TRY(ctx, cudaMemset(c.r, 0, c.ncell * sizeof(float)));
        FSIM_CUDA_TRY(ctx, cudaMemset(c.code, 0, c.ncell * sizeof(uint16_t)));
        FSIM_CUDA_TRY(ctx, cudaMemset(c.kind, 2, c.ncell));
        S.mg.push_back(c);
    }
    if ((long long)S.mg.back().nx * S.mg.back().ny * S.mg.back().nz > MG_BOTTOM_MAX) {
        ctx->err = "multigrid coarsest level too large";
        return FSIM_E_INVALID;
    }
    // cluster for the coarse V-cycle: 16 CTAs where the GPU schedules them, else 8
    S.mg_cluster = 0;
    cudaFuncSetAttribute(k_mg_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize, MG_CLUSTER_SMEM);
    for (int cs : {16, 8}) {
        if (cs > 8 && cudaFuncSetAttribute(k_mg_coarse, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                          cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(MG_CLUSTER_THREADS);
        cfg.dynamicSmemBytes = MG_CLUSTER_SMEM;  // the most a launch asks for
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_mg_coarse, &cfg) == cudaSuccess && nclusters > 0) {
            S.mg_cluster = cs;
            break;
        }
        cudaGetLastError();
    }
    return FSIM_OK;
}

static MGLev mg_lev(const SolverBufs& S, int l, const float* f0, const float* f1, float* x0) {
    const MGLevelBufs& b = S.mg[l];
    MGLev L;
    L.nx = b.nx; L.ny = b.ny; L.nz = b.nz; L.pz = b.pz;
    L.code = b.code;
    L.r = b.r;
    if (l == 0) {
        L.x = x0; L.f = f0; L.f1 = f1;
    } else {
        L.x = b.x; L.f = b.f; L.f1 = nullptr;
    }
    return L;
}

// per-solve: coarse cell kinds and codes from the fine flags
static void mg_setup(fsim_ctx* ctx) {
    SolverBufs& S = ctx->sv;
    cudaStream_t st = ctx->stream;
    for (size_t l = 1; l < S.mg.size(); l++) {
        MGLev F = mg_lev(S, (int)l - 1, nullptr, nullptr, nullptr);
        MGLev Cl = mg_lev(S, (int)l, nullptr, nullptr, nullptr);
        const long long n = S.mg[l].ncell;
        k_mg_coarsen<<<ceil_div(n, 256), 256, 0, st>>>(F, l == 1 ? nullptr : S.mg[l - 1].kind, ctx->flags, Cl,
                                                       S.mg[l].kind);
        k_mg_code<<<ceil_div(n, 256), 256, 0, st>>>(Cl, S.mg[l].kind, S.mg[l].code);
        ctx->launches += 2;
    }
}

// free-surface band sweeps on level l (only the finest level has a band)
static int mg_band_sweeps(const SolverBufs& S, const fsim_params& P, int l) {
    if (l != 0 || P.mg_boundary_sweeps < 0) return 0;
    if (P.mg_boundary_sweeps > 0) return P.mg_boundary_sweeps;
    return S.mg[0].ncell >= MG_BAND_MIN_CELLS ? MG_NB_DEFAULT_BIG : 0;
}

// z = V-cycle(r); r is the current PCG residual (r0 or r1 by device state).
// first_fused: the first level-0 sweep was done by k_update; dot_mode >= 0: the
// last level-0 sweep also computes z.r and the CG scalars (k_red modes).
static void mg_vcycle(fsim_ctx* ctx, const PcgArgs& A, int l, const float* r0, const float* r1, float* z,
                      bool first_fused, int dot_mode) {
    const fsim_params& P = ctx->prm;
    const bool big = ctx->sv.mg[0].ncell >= MG_BAND_MIN_CELLS;
    const int NU0 = P.mg_sweeps > 0 ? P.mg_sweeps : (big ? MG_NU_DEFAULT_BIG : MG_NU_DEFAULT);
    const int NU1 = P.mg_coarse_sweeps > 0 ? P.mg_coarse_sweeps : MG_NU_COARSE_DEFAULT;
    const int NUC = P.mg_cluster_sweeps > 0 ? P.mg_cluster_sweeps : MG_NU_CLUSTER_DEFAULT;
    const int NU = l == 0 ? NU0 : (P.mg_coarse_sweeps > 0 ? NU1 : (l == 1 ? MG_NU_L1_DEFAULT : NU1));
    SolverBufs& S = ctx->sv;
    cudaStream_t st = ctx->stream;
    const int G = S.grid_blocks;
    MGLev L = mg_lev(S, l, r0, r1, z);
    const int last = (int)S.mg.size() - 1;
    if (l == last) {
        launch_pdl(k_mg_bottom, 1, 1024, st, A.st, L);
        ctx->launches += 1;
        return;
    }
    if (l > 0 && S.mg_cluster > 0 && (long long)S.mg[l].ncell <= MG_CLUSTER_CELLS && last - l < MG_MAX_LEVELS) {
        MGChain C{};
        for (int k = l; k <= last; k++) C.lev[k - l] = mg_lev(S, k, nullptr, nullptr, nullptr);
        C.lc = 0;
        C.last = last - l;
        C.nu = NUC;
        C.nu_small = P.mg_cluster_sweeps > 0 ? NUC : MG_NU_SMALL_DEFAULT;
        // the levels from ls on run in shared memory (x, f, r floats + codes per cell)
        C.ls = C.last;
        size_t smem = 0;
        for (int k = C.last; k >= 0; k--) {
            const MGLevelBufs& b = S.mg[l + k];
            const long long n = (long long)b.nx * b.ny * b.nz;
            if (n > MG_SMEM_CELLS) break;
            C.ls = k;
        }
        for (int k = C.ls; k <= C.last; k++) {
            const MGLevelBufs& b = S.mg[l + k];
            const long long n = (long long)b.nx * b.ny * b.nz;
            smem += (size_t)(3 * n + (n + 1) / 2) * sizeof(float);
        }
        // levels lc .. ls-1 as x slabs in the cluster's distributed shared memory
        // when they fit beside rank 0's levels (else they run in global memory)
        size_t slab_floats = 0;
        for (int k = 0; k < C.ls; k++) {
            const MGLevelBufs& b = S.mg[l + k];
            const int P = ceil_div(b.nx, S.mg_cluster);
            const long long m = (long long)P * b.ny * b.nz;
            C.P[k] = P;
            C.off[k] = (int)slab_floats;
            slab_floats += (size_t)((3 * m + (m + 1) / 2 + 3) & ~3ll);
        }
        C.soff = (int)slab_floats;
        const size_t slab_bytes = slab_floats * sizeof(float) + smem;
        C.slab = (C.ls > 0 && slab_bytes <= (size_t)MG_CLUSTER_SMEM) ? 1 : 0;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(S.mg_cluster);
        cfg.blockDim = dim3(MG_CLUSTER_THREADS);
        cfg.dynamicSmemBytes = C.slab ? slab_bytes : smem;
        cfg.stream = st;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = S.mg_cluster;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 2;
        cudaLaunchKernelEx(&cfg, k_mg_coarse, A, C);
        ctx->launches += 1;
        return;
    }
    const int nb = l == 0 ? G : std::min(G, ceil_div(S.mg[l].ncell, 256));
    auto smooth = [&](int color, int first) {
        if (l == 0) launch_pdl(k_mg_smooth<true>, nb, PCG_THREADS, st, A, L, color, first);
        else launch_pdl(k_mg_smooth<false>, nb, PCG_THREADS, st, A, L, color, first);
    };
    for (int k = 0; k < NU; k++) {
        if (k == 0 && l == 0 && first_fused) continue;
        smooth(0, k == 0);
        smooth(1, 0);
        ctx->launches += 2;
    }
    const int NB = mg_band_sweeps(S, P, l);
    auto smooth_band = [&](int color) {
        launch_pdl(k_mg_smooth_bnd, G, PCG_THREADS, st, A, L, (const int4*)S.bnd_quads, (const int*)S.d_nbnd, color);
        ctx->launches += 1;
    };
    for (int k = 0; k < NB; k++) {
        smooth_band(0);
        smooth_band(1);
    }
    if (l == 0) launch_pdl(k_mg_residual<true>, nb, PCG_THREADS, st, A, L);
    else launch_pdl(k_mg_residual<false>, nb, PCG_THREADS, st, A, L);
    MGLev Cl = mg_lev(S, l + 1, nullptr, nullptr, nullptr);
    const int nbc = std::min(G, ceil_div(S.mg[l + 1].ncell, 256));
    launch_pdl(k_mg_restrict, nbc, PCG_THREADS, st, A.st, L, Cl);
    mg_vcycle(ctx, A, l + 1, nullptr, nullptr, nullptr, false, -1);
    if (l == 0) launch_pdl(k_mg_prolong<true>, nb, PCG_THREADS, st, A, L, Cl);
    else launch_pdl(k_mg_prolong<false>, nb, PCG_THREADS, st, A, L, Cl);
    // the pre-smoothing's band sweeps in reverse order (the V-cycle stays symmetric)
    for (int k = 0; k < NB; k++) {
        smooth_band(1);
        smooth_band(0);
    }
    for (int k = 0; k < NU; k++) {
        smooth(1, 0);
        if (l == 0 && k == NU - 1 && dot_mode >= 0)
            launch_pdl(k_mg_smooth_dot, nb, PCG_THREADS, st, A, L, dot_mode);
        else
            smooth(0, 0);
        ctx->launches += 2;
    }
    ctx->launches += 3;
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
    cudaFree(S.brick_xyz); cudaFree(S.d_nactive); cudaFree(S.brick_flag); cudaFree(S.code);
    cudaFree(S.b); cudaFree(S.phi); cudaFree(S.r); cudaFree(S.r64); cudaFree(S.partials);
    cudaFree(S.counter); cudaFree(S.st); cudaFreeHost(S.st_host); cudaFree(S.guess);
    cudaFree(S.bnd_quads); cudaFree(S.d_nbnd);
    for (int k = 0; k < SolverBufs::kIterGraphs; k++)
        if (S.iter_exec[k]) cudaGraphExecDestroy(S.iter_exec[k]);
    for (size_t l = 0; l < S.mg.size(); l++) {
        cudaFree(S.mg[l].r);
        if (l > 0) {
            cudaFree(S.mg[l].kind); cudaFree(S.mg[l].code); cudaFree(S.mg[l].x); cudaFree(S.mg[l].f);
        }
    }
    S = SolverBufs{};
}

// ---- judged initial guess --------------------------------------------------
// ||b - A phi|| (previous pressure) against ||b - A guess||, FP32 per cell and
// FP64 per thread; the last block records which one seeds PCG.
__global__ void __launch_bounds__(PCG_THREADS) k_guess_judge(const PcgArgs a, const float* guess) {
    __shared__ double scratch[32 * 2];
    double acc[2] = {0.0, 0.0};
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        const float ns = (float)code_ns(cc);
        float ap = ns * (float)a.phi[c], ag = ns * guess[c];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if ((cc >> k) & 1) {
                const long long j = c + nb_off(a.B, k);
                ap -= (float)a.phi[j];
                ag -= guess[j];
            }
        const float bc = (float)a.b[c];
        const float rp = bc - ap, rg = bc - ag;
        acc[0] += (double)(rp * rp);
        acc[1] += (double)(rg * rg);
    }
    if (last_block_reduce<2>(acc, 0, a.partials, a.counter, scratch)) {
        if (threadIdx.x == 0) a.st->guess_used = (acc[1] < acc[0]) ? 1 : 0;
    }
}

// r = b - A phi in FP64 on the fluid cells of the active bricks (0 elsewhere):
// the rhs of the correction the previous pressure still needs
__global__ void __launch_bounds__(PCG_THREADS) k_prev_residual(const PcgArgs a, double* r) {
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        const uint16_t cc = a.code[c];
        if (!(cc & CODE_FLUID)) continue;
        double ap = (double)code_ns(cc) * a.phi[c];
#pragma unroll
        for (int k = 0; k < 6; k++)
            if ((cc >> k) & 1) ap -= a.phi[c + nb_off(a.B, k)];
        r[c] = a.b[c] - ap;
    }
}

// guess = phi + correction on the fluid cells of the active bricks
__global__ void __launch_bounds__(PCG_THREADS) k_guess_add_prev(const PcgArgs a, float* guess) {
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        if (a.code[c] & CODE_FLUID) guess[c] = (float)(a.phi[c] + (double)guess[c]);
    }
}

__global__ void __launch_bounds__(PCG_THREADS) k_guess_apply(const PcgArgs a, const float* guess) {
    if (!a.st->guess_used) return;
    const int nact = *a.nactive;
    for (int bk = blockIdx.x; bk < nact; bk += gridDim.x) {
        int x, y, z;
        long long c;
        if (!brick_cell(a.B, a.bxyz[bk], threadIdx.x, x, y, z, c)) continue;
        if (a.code[c] & CODE_FLUID) a.phi[c] = (double)guess[c];
    }
}

template <typename T>
static int run_pcg(fsim_ctx* ctx, PcgArgs& A, Vecs<T> v, int precision, int precond, fsim_step_stats* stats) {
    SolverBufs& S = ctx->sv;
    cudaStream_t st = ctx->stream;
    const int G = S.grid_blocks;
    const bool fold = (precision == FSIM_PREC_MIXED);
    const bool mg = (precond == FSIM_PRECOND_MG) && sizeof(T) == 4;
    int folds = 0;
    auto read_state = [&]() -> int {
        fetch_small(S.st_host, S.st, (int)sizeof(PcgState), st);
        FSIM_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        return FSIM_OK;
    };
    // z = M^-1 r and sigma (mode 0 setup, 1 iteration, 2 after a fold)
    auto precondition = [&](int mode, bool black_done) {
        if (mg) {
            // mode 1: k_update already did the first sweep; the V-cycle ends with z.r
            mg_vcycle(ctx, A, 0, (const float*)(const void*)v.r[0], (const float*)(const void*)v.r[1],
                      (float*)(void*)v.z, mode == 1, mode);
        } else {
            if (!black_done) {
                k_black<T><<<G, PCG_THREADS, 0, st>>>(A, v);
                ctx->launches += 1;
            }
            k_red<T><<<G, PCG_THREADS, 0, st>>>(A, v, mode);
            ctx->launches += 1;
        }
    };
    if (mg) mg_setup(ctx);
    if (mg && mg_band_sweeps(S, ctx->prm, 0) > 0) {
        if (!S.bnd_quads) {
            FSIM_CUDA_TRY(ctx, cudaMalloc(&S.bnd_quads, (size_t)(ctx->g.ncell / 4 + 1) * sizeof(int4)));
            FSIM_CUDA_TRY(ctx, cudaMalloc(&S.d_nbnd, sizeof(int)));
        }
        FSIM_CUDA_TRY(ctx, cudaMemsetAsync(S.d_nbnd, 0, sizeof(int), st));
        k_bnd_list<<<G, PCG_THREADS, 0, st>>>(A, mg_lev(S, 0, nullptr, nullptr, nullptr), S.bnd_quads, S.d_nbnd);
        ctx->launches += 1;
    }
    // initial residual, preconditioned residual, sigma
    k_residual<T><<<G, PCG_THREADS, 0, st>>>(A, v, 1, 1);
    ctx->launches += 1;
    precondition(0, false);
    fsim_record(ctx, EV_PCG_SETUP);
    int rc = read_state();
    if (rc) return rc;
    // one iteration as a CUDA graph (captured once per context and configuration;
    // every kernel reads its varying scalars from the device state)
    auto enqueue_iteration = [&]() {
        if (mg) {
            const MGLev L0 = mg_lev(S, 0, nullptr, nullptr, nullptr);
            Vecs<float> vf = *reinterpret_cast<Vecs<float>*>(&v);
            launch_pdl(k_spmv_q, G, PCG_THREADS, st, A, vf, L0);
            launch_pdl(k_update_q, G, PCG_THREADS, st, A, vf, L0);
        } else {
            k_spmv<T><<<G, PCG_THREADS, 0, st>>>(A, v);
            k_update<T, 1><<<G, PCG_THREADS, 0, st>>>(A, v);
        }
        ctx->launches += 2;
        precondition(1, true);
    };
    const int key = (int)sizeof(T) * 10000000 + (mg ? 1000000 : 0) + ctx->prm.mg_sweeps * 10000 +
                    ctx->prm.mg_coarse_sweeps * 100 + ctx->prm.mg_cluster_sweeps +
                    (ctx->prm.mg_boundary_sweeps + 1) * 100000000;
    int gi = -1;
    for (int k = 0; k < SolverBufs::kIterGraphs; k++)
        if (S.iter_exec[k] && S.iter_key[k] == key) gi = k;
    if (gi < 0) {
        // a free slot, else the least recently used one
        gi = 0;
        for (int k = 0; k < SolverBufs::kIterGraphs; k++) {
            if (!S.iter_exec[k]) { gi = k; break; }
            if (S.iter_used[k] < S.iter_used[gi]) gi = k;
        }
        if (S.iter_exec[gi]) {
            cudaGraphExecDestroy(S.iter_exec[gi]);
            S.iter_exec[gi] = nullptr;
        }
        const long long l0 = ctx->launches;
        cudaGraph_t graph = nullptr;
        FSIM_CUDA_TRY(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        enqueue_iteration();
        FSIM_CUDA_TRY(ctx, cudaStreamEndCapture(st, &graph));
        cudaError_t ie = cudaGraphInstantiate(&S.iter_exec[gi], graph, 0);
        cudaGraphDestroy(graph);
        FSIM_CUDA_TRY(ctx, ie);
        S.iter_key[gi] = key;
        S.iter_kernels[gi] = (int)(ctx->launches - l0);
        ctx->launches = l0;
    }
    S.iter_used[gi] = ++S.iter_clock;
    cudaGraphExec_t iter_exec = S.iter_exec[gi];
    const int iter_kernels = S.iter_kernels[gi];
    double& conv_rate = S.conv_rate[mg ? 1 : 0];
    // Iterations are launched in chunks between host reads of the state.  The
    // chunk is the number of iterations the measured convergence rate (residual
    // norm factor per iteration, carried over from earlier solves) needs to reach
    // the next stop -- the tolerance or the next fold -- so that few iterations
    // are launched past the stop (they exit at once) and few reads are wasted.
    const int chunk_cap = mg ? 16 : 64;
    auto plan = [&]() -> int {
        const PcgState& h = *S.st_host;
        const double rate = conv_rate;
        if (!(rate > 0.0 && rate < 1.0)) return mg ? 2 : 4;
        const double lr = std::log(rate);
        double n = 1e9;
        if (h.tol_mode == FSIM_TOL_ABS_MAX) {
            if (h.rmax > 0.0 && h.tol_abs > 0.0) n = std::log(h.tol_abs / h.rmax) / lr;
        } else if (h.rr > 0.0 && h.tol_rel2 > 0.0) {
            n = 0.5 * std::log(h.tol_rel2 / h.rr) / lr;
        }
        if (fold && h.rr > 0.0 && h.rr_update > 0.0)
            n = std::min(n, 0.5 * std::log(h.fold_drop * h.rr_update / h.rr) / lr);
        return (int)std::min<double>(chunk_cap, std::max(1.0, std::ceil(n)));
    };
    int chunk = plan();
    int it_mark = S.st_host->it;
    double rr_mark = S.st_host->rr;
    while (!S.st_host->done && !S.st_host->nan) {
        for (int k = 0; k < chunk; k++) {
            FSIM_CUDA_TRY(ctx, cudaGraphLaunch(iter_exec, st));
            ctx->launches += iter_kernels;
        }
        if ((rc = read_state())) return rc;
        PcgState& h = *S.st_host;
        if (h.nan) break;
        if (h.it > it_mark && rr_mark > 0.0 && h.rr > 0.0 && h.rr < rr_mark) {
            const double r = std::pow(h.rr / rr_mark, 0.5 / (h.it - it_mark));
            conv_rate = conv_rate > 0.0 ? 0.5 * (conv_rate + r) : r;
        }
        it_mark = h.it;
        rr_mark = h.rr;
        chunk = plan();
        const bool need_fold = fold && (h.need_fold || h.done);
        if (need_fold && !h.skip) {
            // fold the FP32 correction into the FP64 solution, recompute the true
            // residual in FP64, and restart CG from it (s = M^-1 r, beta = 0)
            k_fold<<<G, PCG_THREADS, 0, st>>>(A, (float*)(void*)v.x);
            const int it_before = h.it;
            h.done = 0;
            h.need_fold = 0;
            FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(&S.st->done, &h.done, sizeof(int), cudaMemcpyHostToDevice, st));
            FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(&S.st->need_fold, &h.need_fold, sizeof(int), cudaMemcpyHostToDevice, st));
            k_residual<T><<<G, PCG_THREADS, 0, st>>>(A, v, 0, 0);
            ctx->launches += 2;
            precondition(0, false);
            folds++;
            if ((rc = read_state())) return rc;
            if (!h.done && it_before >= h.max_iters) h.done = 1;
            if (h.done) break;
            it_mark = h.it;
            rr_mark = h.rr;
            chunk = plan();
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
    const bool learned = warm == FSIM_WARM_LEARNED || warm == FSIM_WARM_LEARNED_RESIDUAL;
    if (learned && !ctx->net) {
        ctx->err = "FSIM_WARM_LEARNED / _LEARNED_RESIDUAL need a network (fsim_set_net)";
        return FSIM_E_STATE;
    }
    // back-off: a network whose guesses keep losing to the previous pressure is
    // skipped (not run) for a growing number of solves
    if (learned && ctx->prm.learned_backoff && ctx->learned_skip > 0) {
        ctx->learned_skip--;
        warm = FSIM_WARM_PREVIOUS;
    }
    // a user or learned guess is judged against the previous pressure after setup
    const bool judged = warm == FSIM_WARM_LEARNED || warm == FSIM_WARM_LEARNED_RESIDUAL ||
                        (warm == FSIM_WARM_GUESS && S.have_guess);
    sa.guess = nullptr;
    sa.rhs_override = rhs_override;
    sa.warm = (warm == FSIM_WARM_ZERO) ? FSIM_WARM_ZERO : FSIM_WARM_PREVIOUS;
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
    k_compact_bricks<<<1, 1024, 0, st>>>(S.brick_flag, S.nbricks, S.nby, S.nbz, S.brick_xyz, S.d_nactive);
    ctx->launches += 2;
    fetch_small(&ctx->h_misc[1], S.d_nactive, (int)sizeof(int), st);

    PcgState h{};
    h.tol_mode = tol_mode;
    h.max_iters = max_iters;
    h.tol_abs = tol / scale;
    h.fold_enabled = (precision == FSIM_PREC_MIXED) ? 1 : 0;
    {
        const int d = ctx->prm.refine_digits > 0 ? std::min(ctx->prm.refine_digits, 6) : MIXED_REFINE_DIGITS;
        h.fold_drop = std::pow(10.0, -2.0 * d);  // on r.r
    }
    *S.st_host = h;
    FSIM_CUDA_TRY(ctx, cudaMemcpyAsync(S.st, S.st_host, sizeof(PcgState), cudaMemcpyHostToDevice, st));

    PcgArgs A;
    A.B = B;
    A.bxyz = S.brick_xyz;
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
    A.phi_zero = (warm == FSIM_WARM_ZERO && !judged) ? 1 : 0;

    int rc;
    if (judged) {
        fsim_record(ctx, EV_GUESS0);
        if (warm == FSIM_WARM_LEARNED) {
            const long long l0 = ctx->net->launches;
            rc = net_guess(ctx->net, g, S.code, ctx->flags, S.b, S.guess, st);
            ctx->launches += ctx->net->launches - l0;
            if (rc) {
                ctx->err = std::string("warm-start network: ") + fsim_net_last_error(ctx->net);
                return rc;
            }
        } else if (warm == FSIM_WARM_LEARNED_RESIDUAL) {
            // the network answers the residual of the previous pressure; its answer
            // is added to that pressure (FP64 scratch: the FP64 solver's r buffer)
            if ((rc = alloc_fp64(ctx))) return rc;
            FSIM_CUDA_TRY(ctx, cudaMemsetAsync(S.r64, 0, (size_t)g.ncell * sizeof(double), st));
            k_prev_residual<<<S.grid_blocks, PCG_THREADS, 0, st>>>(A, S.r64);
            const long long l0 = ctx->net->launches;
            rc = net_guess(ctx->net, g, S.code, ctx->flags, S.r64, S.guess, st);
            ctx->launches += ctx->net->launches - l0 + 2;
            if (rc) {
                ctx->err = std::string("warm-start network: ") + fsim_net_last_error(ctx->net);
                return rc;
            }
            k_guess_add_prev<<<S.grid_blocks, PCG_THREADS, 0, st>>>(A, S.guess);
        }
        k_guess_judge<<<S.grid_blocks, PCG_THREADS, 0, st>>>(A, S.guess);
        k_guess_apply<<<S.grid_blocks, PCG_THREADS, 0, st>>>(A, S.guess);
        ctx->launches += 2;
        fsim_record(ctx, EV_GUESS1);
    }
    if (precision == FSIM_PREC_FP64) {
        if ((rc = alloc_fp64(ctx))) return rc;
        const size_t nc = (size_t)g.ncell;
        Vecs<double> v;
        v.r[0] = S.r64; v.r[1] = S.r64 + nc;
        v.s[0] = S.s64; v.s[1] = S.s64 + nc;
        v.z = S.z64; v.q = S.q64;
        v.x = S.phi;
        rc = run_pcg<double>(ctx, A, v, precision, FSIM_PRECOND_RBIC, stats);
    } else {
        const size_t nc = (size_t)g.ncell;
        Vecs<float> v;
        v.r[0] = S.r; v.r[1] = S.r + nc;
        v.s[0] = S.s; v.s[1] = S.s + nc;
        v.z = S.z; v.q = S.q;
        v.x = S.plo;
        rc = run_pcg<float>(ctx, A, v, precision, ctx->prm.precond, stats);
    }
    if (rc) return rc;
    PcgState& hs = *S.st_host;
    if (learned && warm != FSIM_WARM_PREVIOUS && ctx->prm.learned_backoff) {
        if (hs.guess_used) {
            ctx->learned_wait = 0;
        } else {
            ctx->learned_wait = ctx->learned_wait ? std::min(2 * ctx->learned_wait, 64) : 1;
            ctx->learned_skip = ctx->learned_wait;
        }
    }
    if (stats) {
        stats->residual_max = hs.rmax * scale;
        stats->residual_rel = hs.bb > 0 ? sqrt(hs.rr / hs.bb) : 0.0;
        stats->rhs_norm = sqrt(hs.bb) * scale;
        stats->num_active_bricks = ctx->h_misc[1];
        stats->guess_used = judged ? (hs.guess_used ? warm : (warm == FSIM_WARM_ZERO ? 0 : FSIM_WARM_PREVIOUS)) : warm;
        stats->ms_guess = 0.f;
        if (judged && ctx->prm.timing) {
            cudaEventSynchronize(ctx->ev[EV_GUESS1]);
            cudaEventElapsedTime(&stats->ms_guess, ctx->ev[EV_GUESS0], ctx->ev[EV_GUESS1]);
        }
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
