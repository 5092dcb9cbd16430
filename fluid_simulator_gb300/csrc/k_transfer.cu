// k_transfer.cu -- particle <-> grid transfers on cell-sorted particles.
//
// Both kernels work on tiles of cells (one CTA per tile): P2G on PX x PY x PZ,
// G2P on TX x TY x TZ.
//
// P2G (Simulator::p2gTransfer, simulator.cpp:314-352, fused with
// markFluidCellsAndCalculateParticleDensities, simulator.cpp:354-368): the CTA
// owns the faces and cell centres of its tile and computes their final values,
// so no grid accumulator ever goes to global memory and no global atomic is
// used.  Each lane takes one cell of the tile plus its one-cell halo, walks
// that cell's particles (contiguous in the sorted order) and adds their
// trilinear contributions to the tile's shared-memory accumulators; lanes of a
// warp hold distinct cells, so their shared-memory adds do not collide.  The
// CTA then normalises (v / weight if weight > 1e-6, else 0), marks cells that
// hold particles as WATER and writes avgPNum.
//
// G2P (Simulator::g2pTransfer, simulator.cpp:375-418): the CTA stages the
// tile's face velocities plus halo (v2, and v for FLIP) into shared memory
// with TMA tensor loads (cp.async.bulk.tensor, completion on an mbarrier),
// then each thread gathers for one particle of the tile and writes the
// particle into the other particle buffer at its sorted position, which
// applies the cell sort to the particle arrays as a side effect.
#include <cudaTypedefs.h>

#include <algorithm>

#include "fsim_ctx.h"

namespace {

constexpr int TX = 8, TY = 8, TZ = 32;

// G2P staged box: x in [x0-1, x0+TX], y in [y0-1, y0+TY], z in [z0-4, z0+TZ+4)
constexpr int BX = TX + 2, BY = TY + 2, BZ = TZ + 8;
constexpr int BOXN = BX * BY * BZ;
constexpr int G2P_THREADS = 256;

struct P2GArgs {
    ParticleBuf p;
    const uint32_t* perm;
    const int* cstart;
    GridGeom g;
    float* u[3];
    uint8_t* flags;
    float* avg;
    int ntx, nty, ntz;
};

// P2G tile (owned cells) and its one-cell halo: 8x16x16 owned cells, seven
// FP32 shared accumulators per cell (face v and weight per axis, density) =
// 57 KB, two 384-thread CTAs per SM.  Tile shapes measured on the 256^3 APIC
// workload (kernel ms): 8x16x16 4.56, 6x16x16 4.71, 12x12x12 4.73,
// 12x16x16 4.75, 8x12x24 4.79, 8x8x32 4.83, 16x16x8 4.96, 8x16x24 5.03.  A
// tile narrow in x (the slowest axis of the cell order) spans fewer runs of
// sorted particles, and the smaller shared-memory share leaves L1 more room
// for the particle re-reads of the four warp roles.
template <int X, int Y, int Z, int THREADS, int MINB>
struct P2GShape {
    static constexpr int PX = X, PY = Y, PZ = Z, QX = X + 2, QY = Y + 2, QZ = Z + 2;
    static constexpr int PCELLS = X * Y * Z;
    static constexpr int SMEM = 7 * PCELLS * (int)sizeof(float);
    static constexpr int NTHREADS = THREADS, MIN_BLOCKS = MINB;
};
// the default: 8x16x16 tiles (57,344 B), three warp quads per CTA, two CTAs per SM
using P2GFast = P2GShape<8, 16, 16, 384, 2>;
// bit-reproducible (fsim_params.deterministic): one warp quad per CTA, so each
// shared accumulator is added to by a single warp in program order (a warp's
// lanes hold distinct cells: one flush instruction never adds twice to an
// address); 8x8x16 tiles (28,672 B), six CTAs per SM.  5.9 against 4.6 ms at
// 256^3 (8x16x16 tiles with one quad: 8.1 ms).
using P2GDet = P2GShape<8, 8, 16, 128, 6>;

// 1D tent weights of the three cell-centred nodes at relative -0.5, 0.5, 1.5
// (f = position in the cell, 0 <= f < 1): the two nodes the reference's
// trunc-based stencil picks get 1 - |f - node|, the third gets 0.
__device__ __forceinline__ void tent3(float f, float (&w)[3]) {
    w[0] = fmaxf(0.f, 0.5f - f);
    w[1] = 1.f - fabsf(f - 0.5f);
    w[2] = fmaxf(0.f, f - 0.5f);
}

// Warps come in quads over blocks of 32 consecutive tile+halo cells (one cell
// per lane): x faces / y faces / z faces / cell-centre density.  All four walk
// the same particles at about the same time, so the later reads hit L1.  Each
// lane walks its cell's particles once and accumulates, in registers, the
// full 2x3x3 face stencil of its axis (faces of the cells at normal offset -1,
// 0 and transverse offsets -1, 0, +1: the union of getFacesAround's 8-face
// stencils over the cell) or the 3x3x3 stencil of getCellsAround -- the merged
// contribution of all particles of the cell, at most 36 registers -- then adds
// the entries inside the tile to the tile's shared accumulators (lanes hold
// distinct cells, so a warp's adds never collide).  Measured on the 256^3 APIC
// workload (12x16x16 tiles, before the one-ahead loads below): 5.33 ms, against 5.69 ms for warp
// pairs (x + density / y + z, 72 accumulators, 168 registers, a 12x16x32 tile
// and one CTA per SM).
template <bool APIC, int AX, int OW, int OV, int NA>
__device__ __forceinline__ void p2g_face_axis(const float (&f)[3], const float (&wt)[3][3], float va,
                                              const float* cm, float h, float zr, float (&acc)[NA]) {
    constexpr int b = AX == 0 ? 1 : 0, c = AX == 2 ? 1 : 2;  // transverse axes, increasing
    const float wn[2] = {1.f - f[AX], f[AX]};
    float K = va, ka = 0.f, kb = 0.f, kc = 0.f;
    if (APIC) {
        // contribution v_a + c[a] . (face - pos) = K + h (c_a ii + c_b (j - 1/2) + c_c (k - 1/2)),
        // with the z terms scaled by zr = cellD.z / cellD.x (1 except in 2D mode)
        K -= h * (cm[0] * f[0] + cm[1] * f[1] + cm[2] * f[2] * zr);
        ka = h * cm[AX] * (AX == 2 ? zr : 1.f);
        kb = h * cm[b];
        kc = h * cm[c] * (c == 2 ? zr : 1.f);
    }
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            const float wbc = wt[b][j] * wt[c][kk];
            const float cbc = K + kb * ((float)j - 0.5f) + kc * ((float)kk - 0.5f);
#pragma unroll
            for (int ii = 0; ii < 2; ii++) {
                const float w = wn[ii] * wbc;
                const int e = (ii * 3 + j) * 3 + kk;
                acc[OW + e] += w;
                acc[OV + e] += w * (APIC ? cbc + ka * (float)ii : K);
            }
        }
}

template <int AX, int OW, int OV, int NA, class S>
__device__ __forceinline__ void p2g_flush_axis(const float (&acc)[NA], int cx, int cy, int cz, int x0, int y0,
                                               int z0, float* s_vw, float* s_w) {
    constexpr int b = AX == 0 ? 1 : 0, c = AX == 2 ? 1 : 2;
    constexpr int PX = S::PX, PY = S::PY, TZ = S::PZ;
    constexpr int NCELL = PX * PY * TZ;
#pragma unroll
    for (int e = 0; e < 18; e++) {
        if (acc[OW + e] == 0.f) continue;
        int o[3];
        o[AX] = e / 9 - 1;
        o[b] = (e / 3) % 3 - 1;
        o[c] = e % 3 - 1;
        const int lx = cx + o[0] - x0, ly = cy + o[1] - y0, lz = cz + o[2] - z0;
        if (lx < 0 || ly < 0 || lz < 0 || lx >= PX || ly >= PY || lz >= TZ) continue;
        const int li = (lx * PY + ly) * TZ + lz;
        atomicAdd(&s_vw[AX * NCELL + li], acc[OV + e]);
        atomicAdd(&s_w[AX * NCELL + li], acc[OW + e]);
    }
}

template <bool APIC, class S>
__global__ void __launch_bounds__(S::NTHREADS, S::MIN_BLOCKS) k_p2g(const P2GArgs a) {
    constexpr int PX = S::PX, PY = S::PY, PZ = S::PZ, QX = S::QX, QY = S::QY, QZ = S::QZ;
    constexpr int PCELLS = S::PCELLS, P2G_THREADS = S::NTHREADS;
    extern __shared__ float sm[];
    float* s_vw = sm;                // [3][PCELLS]
    float* s_w = sm + 3 * PCELLS;   // [3][PCELLS]
    float* s_avg = sm + 6 * PCELLS;
    for (int k = threadIdx.x; k < 7 * PCELLS; k += blockDim.x) sm[k] = 0.f;
    const int bt = blockIdx.x;
    const int tz = bt % a.ntz, ty = (bt / a.ntz) % a.nty, tx = bt / (a.ntz * a.nty);
    const int x0 = tx * PX, y0 = ty * PY, z0 = tz * PZ;
    __syncthreads();
    const float h = a.g.h, zr = a.g.two_d ? (float)(a.g.hzd * a.g.hinvd) : 1.f;
    const float hinv3[3] = {a.g.hinv, a.g.hinv, a.g.hzinv};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int role = warp & 3;
    const int quads = P2G_THREADS / 128;
    constexpr int HC = QX * QY * QZ;

    for (int blk = warp >> 2; blk * 32 < HC; blk += quads) {
        const int hc = blk * 32 + lane;
        if (hc >= HC) continue;
        const int hz = hc % QZ, hy = (hc / QZ) % QY, hx = hc / (QZ * QY);
        const int cx = x0 - 1 + hx, cy = y0 - 1 + hy, cz = z0 - 1 + hz;
        if (cx < 0 || cy < 0 || cz < 0 || cx >= a.g.nx || cy >= a.g.ny || cz >= a.g.nz) continue;
        const long long cell = gidx(a.g, cx, cy, cz);
        const int beg = a.cstart[cell], end = a.cstart[cell + 1];
        if (beg == end) continue;
        const int cc[3] = {cx, cy, cz};
        float acc[36];
#pragma unroll
        for (int e = 0; e < 36; e++) acc[e] = 0.f;
        // software pipeline: the next particle's index and position are loaded
        // while this one is accumulated (the kernel is latency-bound on these
        // dependent loads; 5.31 -> 4.81 ms at 256^3)
        uint32_t inext = a.perm[beg];
        float pn[3] = {a.p.p[0][inext], a.p.p[1][inext], a.p.p[2][inext]};
        for (int k = beg; k < end; k++) {
            const uint32_t i = inext;
            float f[3];
#pragma unroll
            for (int d = 0; d < 3; d++) f[d] = pn[d] * hinv3[d] - (float)cc[d];
            if (k + 1 < end) {
                inext = a.perm[k + 1];
#pragma unroll
                for (int d = 0; d < 3; d++) pn[d] = a.p.p[d][inext];
            }
            float wt[3][3];
#pragma unroll
            for (int d = 0; d < 3; d++) tent3(f[d], wt[d]);
            if (role == 3) {
#pragma unroll
                for (int ox = 0; ox < 3; ox++)
#pragma unroll
                    for (int oy = 0; oy < 3; oy++) {
                        const float wxy = wt[0][ox] * wt[1][oy];
#pragma unroll
                        for (int oz = 0; oz < 3; oz++) acc[(ox * 3 + oy) * 3 + oz] += wxy * wt[2][oz];
                    }
            } else {
                float cm[3] = {0.f, 0.f, 0.f};
                if (APIC) {
#pragma unroll
                    for (int q = 0; q < 3; q++) cm[q] = a.p.c[3 * role + q][i];
                }
                const float va = a.p.v[role][i];
                if (role == 0) p2g_face_axis<APIC, 0, 0, 18>(f, wt, va, cm, h, zr, acc);
                else if (role == 1) p2g_face_axis<APIC, 1, 0, 18>(f, wt, va, cm, h, zr, acc);
                else p2g_face_axis<APIC, 2, 0, 18>(f, wt, va, cm, h, zr, acc);
            }
        }
        if (role == 3) {
#pragma unroll
            for (int e = 0; e < 27; e++) {
                if (acc[e] == 0.f) continue;
                const int lx = cx + e / 9 - 1 - x0, ly = cy + (e / 3) % 3 - 1 - y0, lz = cz + e % 3 - 1 - z0;
                if (lx < 0 || ly < 0 || lz < 0 || lx >= PX || ly >= PY || lz >= PZ) continue;
                atomicAdd(&s_avg[(lx * PY + ly) * PZ + lz], acc[e]);
            }
        } else if (role == 0) {
            p2g_flush_axis<0, 0, 18, 36, S>(acc, cx, cy, cz, x0, y0, z0, s_vw, s_w);
        } else if (role == 1) {
            p2g_flush_axis<1, 0, 18, 36, S>(acc, cx, cy, cz, x0, y0, z0, s_vw, s_w);
        } else {
            p2g_flush_axis<2, 0, 18, 36, S>(acc, cx, cy, cz, x0, y0, z0, s_vw, s_w);
        }
    }
    __syncthreads();
    for (int lc = threadIdx.x; lc < PCELLS; lc += blockDim.x) {
        const int lz = lc % PZ, ly = (lc / PZ) % PY, lx = lc / (PZ * PY);
        const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
        if (x >= a.g.nx || y >= a.g.ny || z >= a.g.nz) continue;
        const long long cell = gidx(a.g, x, y, z);
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            const float w = s_w[ax * PCELLS + lc];
            a.u[ax][cell] = (w > 1e-6f) ? s_vw[ax * PCELLS + lc] / w : 0.f;
        }
        a.flags[cell] = (a.cstart[cell + 1] > a.cstart[cell]) ? C_WATER : C_AIR;
        a.avg[cell] = s_avg[lc];
    }
}

// ---- TMA / mbarrier helpers (inline PTX) ------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
    return ok != 0;
}

struct G2PArgs {
    ParticleBuf src, dst;
    const uint32_t* perm;
    const int* cstart;
    GridGeom g;
    int ntx, nty, ntz;
    float fr;          // flipRatio
    float pic_w;       // (1 - flipRatio) evaluated in float, as the reference does
    int ids;
    int move_c;        // PIC/FLIP: carry C along the permutation
    unsigned* err;
};

// MODE: 0 PIC, 1 FLIP, 2 APIC
template <int MODE>
__global__ void __launch_bounds__(G2P_THREADS) k_g2p(const G2PArgs a, const __grid_constant__ CUtensorMap m0,
                                                     const __grid_constant__ CUtensorMap m1,
                                                     const __grid_constant__ CUtensorMap m2,
                                                     const __grid_constant__ CUtensorMap m3,
                                                     const __grid_constant__ CUtensorMap m4,
                                                     const __grid_constant__ CUtensorMap m5) {
    extern __shared__ __align__(128) unsigned char smraw[];
    float* sv2 = reinterpret_cast<float*>(smraw);  // [3][BOXN]
    float* su = sv2 + 3 * BOXN;                    // [3][BOXN] (FLIP)
    __shared__ __align__(8) uint64_t mbar;
    __shared__ int seg_beg[TX * TY];
    __shared__ int seg_pre[TX * TY + 1];

    const int bt = blockIdx.x;
    const int tz = bt % a.ntz, ty = (bt / a.ntz) % a.nty, tx = bt / (a.ntz * a.nty);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    if (threadIdx.x == 0) {
        mbar_init(&mbar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nmaps = (MODE == 1) ? 6 : 3;
        mbar_expect_tx(&mbar, (unsigned)(nmaps * BOXN * sizeof(float)));
        tma_load_3d(sv2 + 0 * BOXN, &m0, z0 - 4, y0 - 1, x0 - 1, &mbar);
        tma_load_3d(sv2 + 1 * BOXN, &m1, z0 - 4, y0 - 1, x0 - 1, &mbar);
        tma_load_3d(sv2 + 2 * BOXN, &m2, z0 - 4, y0 - 1, x0 - 1, &mbar);
        if (MODE == 1) {
            tma_load_3d(su + 0 * BOXN, &m3, z0 - 4, y0 - 1, x0 - 1, &mbar);
            tma_load_3d(su + 1 * BOXN, &m4, z0 - 4, y0 - 1, x0 - 1, &mbar);
            tma_load_3d(su + 2 * BOXN, &m5, z0 - 4, y0 - 1, x0 - 1, &mbar);
        }
    }
    // particle segments of the tile: one contiguous run per (x, y) row
    if (threadIdx.x < 64) {
        const int r = threadIdx.x;
        const int x = x0 + r / TY, y = y0 + r % TY;
        int beg = 0, len = 0;
        if (x < a.g.nx && y < a.g.ny) {
            const long long base = gidx(a.g, x, y, 0);
            const int ze = min(z0 + TZ, a.g.pz);
            beg = a.cstart[base + z0];
            len = a.cstart[base + ze] - beg;
        }
        seg_beg[r] = beg;
        int x_incl = len;
        const int lane = r & 31;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y2 = __shfl_up_sync(0xffffffffu, x_incl, o);
            if (lane >= o) x_incl += y2;
        }
        seg_pre[r + 1] = x_incl;  // warp-local inclusive prefix; fixed below
        if (r == 0) seg_pre[0] = 0;
    }
    __syncthreads();
    if (threadIdx.x >= 32 && threadIdx.x < 64) seg_pre[threadIdx.x + 1] += seg_pre[32];
    __syncthreads();
    const int total = seg_pre[TX * TY];
    // sorted slot of the tile's j-th particle: its row by binary search for a
    // thread's first particle, then by stepping forward from the previous row
    // (a thread's particles come in increasing j, a row is ~TZ*8 particles)
    int row = 0;
    auto slot_of = [&](int j) {
        int lo = 0, hi = TX * TY - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (seg_pre[mid] <= j) lo = mid; else hi = mid - 1;
        }
        row = lo;
        return seg_beg[lo] + (j - seg_pre[lo]);
    };
    auto slot_next = [&](int j) {
        while (row + 1 < TX * TY && seg_pre[row + 1] <= j) row++;
        return seg_beg[row] + (j - seg_pre[row]);
    };
    // software pipeline: each thread's next particle (slot, index, position) is
    // loaded one iteration ahead; the first one while the grid tile is in flight
    int kn = 0;
    uint32_t in = 0;
    float pn[3] = {0.f, 0.f, 0.f};
    if ((int)threadIdx.x < total) {
        kn = slot_of(threadIdx.x);
        in = a.perm[kn];
        pn[0] = a.src.p[0][in]; pn[1] = a.src.p[1][in]; pn[2] = a.src.p[2][in];
    }
    // wait for the staged grid (bounded: about 2^31 cycles, then report and leave;
    // the leave decision is made for the whole CTA at once, after a second bounded
    // wait for the copies still in flight)
    {
        const long long t0 = clock64();
        bool ok = false;
        while (!(ok = mbar_try_wait(&mbar, 0))) {
            if (clock64() - t0 > (1ll << 31)) break;
        }
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, FSIM_DERR_TMA_TIMEOUT);
                const long long t1 = clock64();
                while (!mbar_try_wait(&mbar, 0) && clock64() - t1 < (1ll << 31)) {
                }
            }
            __syncthreads();
            return;
        }
    }
    const float hinv = a.g.hinv, hzinv = a.g.hzinv;
    for (int j = threadIdx.x; j < total; j += blockDim.x) {
        const int k = kn;
        const uint32_t i = in;
        const float px = pn[0], py = pn[1], pz = pn[2];
        if (j + (int)blockDim.x < total) {
            kn = slot_next(j + blockDim.x);
            in = a.perm[kn];
            pn[0] = a.src.p[0][in]; pn[1] = a.src.p[1][in]; pn[2] = a.src.p[2][in];
        }
        const float g[3] = {px * hinv, py * hinv, pz * hzinv};
        float vnew[3];
        float cnew[9];
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            int b[3];
            float d0[3];
#pragma unroll
            for (int dd = 0; dd < 3; dd++) {
                const float off = (dd == ax) ? 0.f : 0.5f;
                b[dd] = (int)(g[dd] - off) - (dd == ax ? 1 : 0);
                d0[dd] = g[dd] - ((float)b[dd] + (dd == ax ? 1.f : 0.5f));
            }
            // shared-box coordinates of the stencil corner
            const int sx = b[0] - (x0 - 1), sy = b[1] - (y0 - 1), sz = b[2] - (z0 - 4);
            // 1D weights and trilinearInterpollGradient signs (util/interpolation.h:21-35)
            // of the two nodes per dimension
            float w1[3][2], sg[3][2];
#pragma unroll
            for (int dd = 0; dd < 3; dd++)
#pragma unroll
                for (int o = 0; o < 2; o++) {
                    const float d = d0[dd] - o;
                    w1[dd][o] = 1.f - fabsf(d);
                    sg[dd][o] = d > 0.f ? -1.f : 1.f;
                }
            if (MODE == 2 && a.g.two_d) {
                // 2D particles sit on the z node plane, where the sign flips: take it
                // from the FP64 offset as the reference does (0.15f * 10 rounds to
                // exactly 1.5 in FP32, 6e-8 above it in FP64)
#pragma unroll
                for (int o = 0; o < 2; o++) {
                    const double e =
                        ((double)pz - ((double)(b[2] + o) + (ax == 2 ? 1.0 : 0.5)) * a.g.hzd) * a.g.hzinvd;
                    sg[2][o] = e > 0.0 ? -1.f : 1.f;
                }
            }
            // The trilinear sums factor by dimension: contract the 2x2x2 corner
            // values along z, then y, then x, with the 1-D weights w and the signed
            // gradient factors g = sign / h (trilinearInterpoll and
            // trilinearInterpollGradient summed over the eight corners, in half
            // the arithmetic of a corner-by-corner sum).
            float gx[2], gy[2], gz[2];
#pragma unroll
            for (int o = 0; o < 2; o++) {
                gx[o] = sg[0][o] * hinv;
                gy[o] = sg[1][o] * hinv;
                gz[o] = sg[2][o] * hzinv;
            }
            float A[2][2], Bz[2][2], Fz[2][2];
#pragma unroll
            for (int ox = 0; ox < 2; ox++)
#pragma unroll
                for (int oy = 0; oy < 2; oy++) {
                    const int si = ((sx + ox) * BY + (sy + oy)) * BZ + sz;
                    const float va = sv2[ax * BOXN + si], vb = sv2[ax * BOXN + si + 1];
                    A[ox][oy] = w1[2][0] * va + w1[2][1] * vb;
                    if (MODE == 2) Bz[ox][oy] = gz[0] * va + gz[1] * vb;
                    if (MODE == 1)
                        Fz[ox][oy] = w1[2][0] * (va - su[ax * BOXN + si]) + w1[2][1] * (vb - su[ax * BOXN + si + 1]);
                }
            float P[2], Gy[2], Q[2], Fy[2];
#pragma unroll
            for (int ox = 0; ox < 2; ox++) {
                P[ox] = w1[1][0] * A[ox][0] + w1[1][1] * A[ox][1];
                if (MODE == 2) {
                    Gy[ox] = gy[0] * A[ox][0] + gy[1] * A[ox][1];
                    Q[ox] = w1[1][0] * Bz[ox][0] + w1[1][1] * Bz[ox][1];
                }
                if (MODE == 1) Fy[ox] = w1[1][0] * Fz[ox][0] + w1[1][1] * Fz[ox][1];
            }
            const float pic = w1[0][0] * P[0] + w1[0][1] * P[1];
            float flip = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
            if (MODE == 1) flip = w1[0][0] * Fy[0] + w1[0][1] * Fy[1];
            if (MODE == 2) {
                c0 = gx[0] * P[0] + gx[1] * P[1];
                c1 = w1[0][0] * Gy[0] + w1[0][1] * Gy[1];
                c2 = w1[0][0] * Q[0] + w1[0][1] * Q[1];
            }
            if (MODE == 0) vnew[ax] = pic;
            if (MODE == 1) vnew[ax] = pic * a.pic_w + (flip + a.src.v[ax][i]) * a.fr;
            if (MODE == 2) {
                vnew[ax] = pic;
                cnew[3 * ax] = c0;
                cnew[3 * ax + 1] = c1;
                cnew[3 * ax + 2] = c2;
            }
        }
        if (a.g.two_d) {
            // 2D mode (simulator.cpp:382-385): v.z = 0 and the z row of C is left as it was
            vnew[2] = 0.f;
            if (MODE == 2) {
#pragma unroll
                for (int q = 6; q < 9; q++) cnew[q] = a.src.c[q][i];
            }
        }
        a.dst.p[0][k] = px;
        a.dst.p[1][k] = py;
        a.dst.p[2][k] = pz;
#pragma unroll
        for (int ax = 0; ax < 3; ax++) a.dst.v[ax][k] = vnew[ax];
        if (MODE == 2) {
#pragma unroll
            for (int q = 0; q < 9; q++) a.dst.c[q][k] = cnew[q];
        } else if (a.move_c) {
#pragma unroll
            for (int q = 0; q < 9; q++) a.dst.c[q][k] = a.src.c[q][i];
        }
        if (a.ids) a.dst.id[k] = a.src.id[i];
    }
}

}  // namespace

namespace {
template <class S>
cudaError_t launch_p2g_shape(P2GArgs a, bool apic, cudaStream_t stream) {
    a.ntx = ceil_div(a.g.nx, S::PX);
    a.nty = ceil_div(a.g.ny, S::PY);
    a.ntz = ceil_div(a.g.nz, S::PZ);
    const int nb = a.ntx * a.nty * a.ntz;
    cudaError_t e = set_smem_limit((const void*)(apic ? k_p2g<true, S> : k_p2g<false, S>), S::SMEM);
    if (e != cudaSuccess) return e;
    if (apic)
        k_p2g<true, S><<<nb, S::NTHREADS, S::SMEM, stream>>>(a);
    else
        k_p2g<false, S><<<nb, S::NTHREADS, S::SMEM, stream>>>(a);
    return cudaGetLastError();
}
}  // namespace

void launch_p2g(fsim_ctx* ctx) {
    P2GArgs a;
    a.p = ctx->buf[ctx->cur];
    a.perm = ctx->perm;
    a.cstart = ctx->cstart;
    a.g = ctx->g;
    for (int k = 0; k < 3; k++) a.u[k] = ctx->u[k];
    a.flags = ctx->flags;
    a.avg = ctx->avg;
    ctx->launches += 1;
    const bool apic = ctx->prm.transfer == FSIM_APIC;
    if (ctx->prm.deterministic) launch_p2g_shape<P2GDet>(a, apic, ctx->stream);
    else launch_p2g_shape<P2GFast>(a, apic, ctx->stream);
}

// P2G on caller-provided buffers (used by the allocation-free entry point in
// fsim_static.cu); the default kernel of launch_p2g.
cudaError_t launch_p2g_raw(ParticleBuf p, const uint32_t* perm, const int* cstart, const GridGeom& g,
                           float* const u[3], uint8_t* flags, float* avg, bool apic, cudaStream_t stream) {
    P2GArgs a;
    a.p = p;
    a.perm = perm;
    a.cstart = cstart;
    a.g = g;
    for (int k = 0; k < 3; k++) a.u[k] = u[k];
    a.flags = flags;
    a.avg = avg;
    return launch_p2g_shape<P2GFast>(a, apic, stream);
}

// TMA descriptors of the six face arrays (v2 x/y/z, v x/y/z): 3D tensors
// (z innermost, padded pitch pz), box BZ x BY x BX floats, zero fill outside.
bool make_tensor_maps(fsim_ctx* ctx) {
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&encode, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || encode == nullptr) {
        ctx->err = "cuTensorMapEncodeTiled unavailable";
        return false;
    }
    const GridGeom& g = ctx->g;
    cuuint64_t dims[3] = {(cuuint64_t)g.pz, (cuuint64_t)g.ny, (cuuint64_t)g.nx};
    cuuint64_t strides[2] = {(cuuint64_t)g.pz * 4, (cuuint64_t)g.pz * g.ny * 4};
    cuuint32_t box[3] = {BZ, BY, BX};
    cuuint32_t estr[3] = {1, 1, 1};
    float* arrays[6] = {ctx->v2[0], ctx->v2[1], ctx->v2[2], ctx->u[0], ctx->u[1], ctx->u[2]};
    for (int k = 0; k < 6; k++) {
        CUresult r = encode(&ctx->tmap[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, arrays[k], dims, strides,
                            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            ctx->err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
            return false;
        }
    }
    ctx->tmap_ok = true;
    return true;
}

int launch_g2p(fsim_ctx* ctx) {
    const GridGeom& g = ctx->g;
    G2PArgs a;
    a.src = ctx->buf[ctx->cur];
    a.dst = ctx->buf[1 - ctx->cur];
    a.perm = ctx->perm;
    a.cstart = ctx->cstart;
    a.g = g;
    a.ntx = ceil_div(g.nx, TX);
    a.nty = ceil_div(g.ny, TY);
    a.ntz = ceil_div(g.nz, TZ);
    a.fr = ctx->prm.flip_ratio;
    a.pic_w = 1.0f - ctx->prm.flip_ratio;
    a.ids = ctx->prm.track_ids ? 1 : 0;
    a.move_c = 1;
    a.err = ctx->d_err;
    const int nb = a.ntx * a.nty * a.ntz;
    const int mode = ctx->prm.transfer;
    ctx->launches += 1;
    const size_t smem = (size_t)((mode == FSIM_FLIP) ? 6 : 3) * BOXN * sizeof(float);
    set_smem_limit((const void*)k_g2p<0>, 3 * BOXN * 4);
    set_smem_limit((const void*)k_g2p<1>, 6 * BOXN * 4);
    set_smem_limit((const void*)k_g2p<2>, 3 * BOXN * 4);
    const CUtensorMap* m = ctx->tmap;
    if (mode == FSIM_PIC)
        k_g2p<0><<<nb, G2P_THREADS, smem, ctx->stream>>>(a, m[0], m[1], m[2], m[3], m[4], m[5]);
    else if (mode == FSIM_FLIP)
        k_g2p<1><<<nb, G2P_THREADS, smem, ctx->stream>>>(a, m[0], m[1], m[2], m[3], m[4], m[5]);
    else
        k_g2p<2><<<nb, G2P_THREADS, smem, ctx->stream>>>(a, m[0], m[1], m[2], m[3], m[4], m[5]);
    return 0;
}
