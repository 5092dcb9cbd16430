// k_conv.cu -- convolutions of the pressure warm-start network on the
// 5th-generation tensor cores (tcgen05, TMEM accumulators, TMA operands).
//
// Tensors are BF16 in NDHWC order ([n][d][h][w][c], c fastest).  Weights are
// BF16 [tap][cout][cin] (tap = (kd*3 + kh)*3 + kw for 3x3x3, a single tap for
// the pointwise convolutions).  Accumulation is FP32.
//
// Forward / input-gradient kernels: implicit GEMM
//   D[m, n] = sum_{tap, c} X[voxel(m) + off(tap), c] * W[tap, n, c]
// over output tiles of 8 (w) x 16 (h) x 4 (d) voxels and NT output channels:
// k_conv_pers (3x3x3 layers) is persistent, one CTA per SM walking the tiles
// with warp-specialized roles (described at the kernel); k_conv_mma (the
// pointwise down-convolutions) gives each CTA one tile.  Per 16-channel chunk
// of the input a CTA loads ONE halo box of the
// input (10 x 18 x 6 voxels for 3x3x3, zero-filled outside the volume, which
// is the padding) and the chunk's weights for all taps with TMA, in the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix,
// the two 8-channel halves of the chunk in separate planes).  Every tap is then
// one tcgen05.mma (M = 128 voxels of one d-plane, N = NT, K = 16) whose A
// descriptor simply starts at the shifted halo row: row groups of 8 voxels are
// 16-byte rows, so a shift by (kw, kh, kd) is a start offset of
// ((kd*18 + kh)*10 + kw) * 16 bytes.  The four d-planes accumulate into four
// TMEM column blocks.  Input-gradient (dgrad) is the same kernel on the output
// gradient with the per-tap transposed weights [tap][cin][cout] read at tap
// 26 - t.  The epilogue reads TMEM with tcgen05.ld, adds the bias, applies
// ReLU or a ReLU-derivative mask, and stores BF16 at a channel stride/offset
// (so encoder outputs land directly in their concatenation slice).
//
// Weight-gradient kernel (k_conv_wgrad): D[(tap, c), n] = sum_v X[v + off(tap), c]
// * G[v, n] with K = voxels.  Threads stage the shifted input transposed into
// the K-major layout (16 voxels per step) with plain loads, a proxy fence
// makes the stores visible to the tensor core, and one thread issues the
// MMAs; the FP32 result is added to the gradient with atomics.
//
// Every wait is bounded; a timeout sets an error bit, waits (bounded) for the
// MMAs already issued, frees TMEM and returns.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "fsim_ctx.h"
#include "fsim_net.h"

namespace {

constexpr int TW = 8, TH = 16, TD = 4;  // output tile (w, h, d); M = TW*TH = 128 per plane
constexpr int CONV_THREADS = 128;
constexpr int SMEM_LIMIT = 227 * 1024 - 1024;  // opt-in maximum minus room for static shared memory
constexpr long long SPIN_LIMIT = 1ll << 31;  // clock cycles, about one second

__device__ __forceinline__ unsigned s32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(s32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned phase) {
    const long long t0 = clock64();
    while (!mbar_try(bar, phase))
        if (clock64() - t0 > SPIN_LIMIT) return false;
    return true;
}
__device__ __forceinline__ void tma_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                       uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(s32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(s32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(s32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(s32(bar))
        : "memory");
}

// tcgen05 shared-memory matrix descriptor, K-major, no swizzle: core matrices
// of 8 rows x 16 bytes; lbo = byte distance between the two K halves, sbo =
// byte distance between 8-row groups.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version
    return d;                // base offset 0, layout 0 = no swizzle
}
// instruction descriptor: D FP32, A and B BF16, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, int ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t base, int ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__host__ __device__ constexpr int tmem_cols(int n) {
    return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512;
}

__device__ __forceinline__ bool bf16_pos(unsigned short bits) { return !(bits & 0x8000u) && bits != 0; }

// ---------------------------------------------------------------------------
// forward / input-gradient
// ---------------------------------------------------------------------------
template <int TAPS>
struct Halo {
    static constexpr int H = TAPS == 27 ? 1 : 0;
    static constexpr int AW = TW + 2 * H, AH = TH + 2 * H, AD = TD + 2 * H;
    static constexpr int ROWS = AW * AH * AD;
    static constexpr int KC = ROWS * 16;  // bytes of one 8-channel half
    static constexpr int A_BYTES = 2 * KC;
};

struct MmaArgs {
    int n, d, h, w;      // volume (input and output have the same size)
    int cin, cout, nt;   // nt = output channels per CTA
    int tiles_w, tiles_h, tiles_d, ntiles;
    int stages;
    int flip;            // weights read at tap 26 - t (input gradient)
    const float* bias;   // [cout] or null
    int relu;
    const __nv_bfloat16* mask;  // ReLU-derivative mask (out *= mask > 0) or null
    int ms, mo;          // mask channel stride / offset
    __nv_bfloat16* y;
    int ys, yo;          // output channel stride / offset
    unsigned* err;
};

template <int TAPS>
__global__ void __launch_bounds__(CONV_THREADS) k_conv_mma(const MmaArgs a, const __grid_constant__ CUtensorMap tx,
                                                           const __grid_constant__ CUtensorMap tw) {
    using G = Halo<TAPS>;
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 127) & ~(uintptr_t)127);
    __shared__ __align__(8) uint64_t full[3], empty[3], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;

    long long t = blockIdx.x;
    const int nti = (int)(t % a.ntiles);
    t /= a.ntiles;
    const int bw = (int)(t % a.tiles_w);
    t /= a.tiles_w;
    const int bh = (int)(t % a.tiles_h);
    t /= a.tiles_h;
    const int bd = (int)(t % a.tiles_d);
    const int nb = (int)(t / a.tiles_d);
    const int w0 = bw * TW, h0 = bh * TH, d0 = bd * TD, n0 = nti * a.nt;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ncols = tmem_cols(TD * a.nt);
    const int B_KC = TAPS * a.nt * 16;
    const int stage_bytes = G::A_BYTES + 2 * B_KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    if (warp == 0) tmem_alloc(&tmem_base, ncols);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;

    const int nchunk = a.cin >> 4;
    if (threadIdx.x == 0) {
        const uint32_t idesc = idesc_bf16(a.nt);
        const unsigned tx_bytes = (unsigned)stage_bytes;
        auto issue = [&](int k) {
            const int s = k % a.stages;
            unsigned char* st = sm + s * stage_bytes;
            mbar_expect_tx(&full[s], tx_bytes);
#pragma unroll
            for (int kc = 0; kc < 2; kc++) {
                tma_5d(st + kc * G::KC, &tx, k * 16 + kc * 8, w0 - G::H, h0 - G::H, d0 - G::H, nb, &full[s]);
                tma_3d(st + G::A_BYTES + kc * B_KC, &tw, k * 16 + kc * 8, n0, 0, &full[s]);
            }
        };
        bool ok = true;
        const int pre = nchunk < a.stages ? nchunk : a.stages;
        for (int k = 0; k < pre; k++) issue(k);
        int issued = pre, consumed = 0;
        for (int k = 0; k < nchunk; k++) {
            const int s = k % a.stages;
            if (!mbar_wait(&full[s], (unsigned)((k / a.stages) & 1))) { ok = false; break; }
            consumed = k + 1;
            fence_after();
            const uint32_t abase = s32(sm + s * stage_bytes);
            const uint32_t bbase = abase + G::A_BYTES;
#pragma unroll 1
            for (int tap = 0; tap < TAPS; tap++) {
                const int kd = tap / 9, kh = (tap / 3) % 3, kw = tap % 3;
                const int wt = a.flip ? TAPS - 1 - tap : tap;
                const uint64_t bdesc = sdesc(bbase + (uint32_t)(wt * a.nt * 16), (uint32_t)B_KC, 128);
#pragma unroll
                for (int zp = 0; zp < TD; zp++) {
                    const int row = ((zp + kd) * G::AH + kh) * G::AW + kw;
                    const uint64_t adesc =
                        sdesc(abase + (uint32_t)(row * 16), (uint32_t)G::KC, (uint32_t)(G::AW * 16));
                    mma_bf16(tmem + (uint32_t)(zp * a.nt), adesc, bdesc, idesc, (k > 0 || tap > 0) ? 1u : 0u);
                }
            }
            mma_commit(&empty[s]);
            if (k + a.stages < nchunk) {
                if (!mbar_wait(&empty[s], (unsigned)((k / a.stages) & 1))) { ok = false; break; }
                issue(k + a.stages);
                issued++;
            }
        }
        mma_commit(&done);
        if (!ok) {
            // let the copies still in flight land before the CTA's shared memory goes away
            for (int k = consumed; k < issued; k++) mbar_wait(&full[k % a.stages], (unsigned)((k / a.stages) & 1));
            s_fail = 1;
            atomicOr(a.err, 1u);
        }
    }
    __syncthreads();
    const bool ok = mbar_wait(&done, 0);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(a.err, 2u);
    } else if (!s_fail) {
        fence_after();
        const int m = warp * 32 + lane;
        const int vw = w0 + (m & 7), vh = h0 + (m >> 3);
#pragma unroll 1
        for (int zp = 0; zp < TD; zp++) {
            const int vd = d0 + zp;
            const bool inside = vw < a.w && vh < a.h && vd < a.d;
            const long long vox = (((long long)nb * a.d + vd) * a.h + vh) * a.w + vw;
#pragma unroll 1
            for (int c0 = 0; c0 < a.nt; c0 += 16) {
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(zp * a.nt + c0), r);
                if (!inside) continue;
                const int ch = n0 + c0;
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
                if (a.bias) {
#pragma unroll
                    for (int j = 0; j < 16; j++) v[j] += a.bias[ch + j];
                }
                if (a.relu) {
#pragma unroll
                    for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j], 0.f);
                }
                if (a.mask) {
                    const uint4* mp = reinterpret_cast<const uint4*>(a.mask + vox * a.ms + a.mo + ch);
                    uint4 mv[2] = {mp[0], mp[1]};
                    const unsigned short* mb = reinterpret_cast<const unsigned short*>(mv);
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        if (!bf16_pos(mb[j])) v[j] = 0.f;
                }
                __align__(16) __nv_bfloat162 o[8];
#pragma unroll
                for (int j = 0; j < 8; j++) o[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                uint4* dst = reinterpret_cast<uint4*>(a.y + vox * a.ys + a.yo + ch);
                dst[0] = reinterpret_cast<const uint4*>(o)[0];
                dst[1] = reinterpret_cast<const uint4*>(o)[1];
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, ncols);
}

// ---------------------------------------------------------------------------
// forward / input-gradient of the 3x3x3 layers: persistent, warp-specialized
// ---------------------------------------------------------------------------
// One CTA per SM walks the output tiles t = blockIdx.x, + gridDim.x, ...  Warp
// 0 (one thread) streams (tile, 16-channel chunk) items into a ring of shared
// memory stages with TMA, warp 1 (one thread) issues each item's 108 MMAs into
// one of two TMEM accumulators, and warps 2-5 drain the other accumulator
// (bias, ReLU or mask, BF16 stores) while the next tile accumulates, so loads,
// MMAs and the epilogue of neighbouring tiles overlap instead of running one
// after the other in every CTA.  When the layer has one N tile and its
// weights fit beside two stages, all chunks' weights are loaded once and stay
// resident; otherwise each stage carries its chunk's weights as above.
// Every wait is bounded; a timeout (or a role that gave up) makes all roles
// stop, the copies in flight land, the issued MMAs finish, TMEM is freed.
constexpr int PERS_THREADS = 192;
constexpr int PERS_MAX_STAGES = 4;

struct PersArgs {
    MmaArgs m;
    int total_tiles;  // tiles_w * tiles_h * tiles_d * n * ntiles
    int wres;         // weights of all chunks resident in shared memory
    int stage_bytes;  // halo box (plus the chunk's weights when not resident)
    int ncols;        // TMEM columns of one accumulator
};

struct TileAt {
    int w0, h0, d0, nb, n0;
};

__device__ __forceinline__ TileAt tile_at(const MmaArgs& a, int t) {
    TileAt c;
    const int nti = t % a.ntiles;
    t /= a.ntiles;
    c.w0 = (t % a.tiles_w) * TW;
    t /= a.tiles_w;
    c.h0 = (t % a.tiles_h) * TH;
    t /= a.tiles_h;
    c.d0 = (t % a.tiles_d) * TD;
    c.nb = t / a.tiles_d;
    c.n0 = nti * a.nt;
    return c;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s32(bar)) : "memory");
}
// bounded wait that also gives up once another role has stopped
__device__ __forceinline__ bool mbar_wait_ab(uint64_t* bar, unsigned phase, volatile int* stop, unsigned* err) {
    const long long t0 = clock64();
    while (!mbar_try(bar, phase)) {
        if (*stop) return false;
        if (clock64() - t0 > SPIN_LIMIT) {
            *stop = 1;
            atomicOr(err, 1u);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__global__ void __launch_bounds__(PERS_THREADS, 1) k_conv_pers(const PersArgs p, const __grid_constant__ CUtensorMap tx,
                                                                const __grid_constant__ CUtensorMap tw) {
    using G = Halo<27>;
    const MmaArgs& a = p.m;
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 127) & ~(uintptr_t)127);
    __shared__ __align__(8) uint64_t full[PERS_MAX_STAGES], empty[PERS_MAX_STAGES], acc_full[2], acc_empty[2];
    __shared__ __align__(8) uint64_t wfull, done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_stop, s_issued, s_consumed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int S = a.stages;
    const int nchunk = a.cin >> 4;
    const int B_KC = 27 * a.nt * 16;
    unsigned char* wbase = sm + S * p.stage_bytes;
    const int my_tiles = (int)blockIdx.x < p.total_tiles ? (p.total_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int items = my_tiles * nchunk;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        mbar_init(&wfull, 1);
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_stop = 0;
        s_issued = 0;
        s_consumed = 0;
    }
    if (warp == 0) tmem_alloc(&tmem_base, 2 * p.ncols);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;
    volatile int* stop = &s_stop;

    if (warp == 0) {
        if (lane == 0) {
            if (p.wres) {
                mbar_expect_tx(&wfull, (unsigned)(nchunk * 2 * B_KC));
                for (int k = 0; k < nchunk; k++)
                    for (int kc = 0; kc < 2; kc++) tma_3d(wbase + (k * 2 + kc) * B_KC, &tw, k * 16 + kc * 8, 0, 0, &wfull);
            }
            int issued = 0;
            for (int j = 0; j < items; j++) {
                const int s = j % S;
                if (j >= S && !mbar_wait_ab(&empty[s], (unsigned)(((j / S) - 1) & 1), stop, a.err)) break;
                const TileAt c = tile_at(a, (int)blockIdx.x + (j / nchunk) * (int)gridDim.x);
                const int k = j % nchunk;
                unsigned char* st = sm + s * p.stage_bytes;
                mbar_expect_tx(&full[s], (unsigned)p.stage_bytes);
#pragma unroll
                for (int kc = 0; kc < 2; kc++) {
                    tma_5d(st + kc * G::KC, &tx, k * 16 + kc * 8, c.w0 - 1, c.h0 - 1, c.d0 - 1, c.nb, &full[s]);
                    if (!p.wres) tma_3d(st + G::A_BYTES + kc * B_KC, &tw, k * 16 + kc * 8, c.n0, 0, &full[s]);
                }
                issued = j + 1;
            }
            s_issued = issued;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(a.nt);
            bool ok = !p.wres || mbar_wait_ab(&wfull, 0, stop, a.err);
            int consumed = 0;
            for (int j = 0; ok && j < items; j++) {
                const int s = j % S, ti = j / nchunk, k = j % nchunk, buf = ti & 1;
                if (!mbar_wait_ab(&full[s], (unsigned)((j / S) & 1), stop, a.err)) break;
                consumed = j + 1;
                if (k == 0 && ti >= 2 && !mbar_wait_ab(&acc_empty[buf], (unsigned)(((ti >> 1) - 1) & 1), stop, a.err))
                    break;
                fence_after();
                const uint32_t abase = s32(sm + s * p.stage_bytes);
                const uint32_t bbase = p.wres ? s32(wbase + k * 2 * B_KC) : abase + G::A_BYTES;
                // The 108 MMAs are unrolled with their descriptors formed by
                // adding to two base descriptors (the start-address field is
                // the byte address / 16, so a shift by `row` halo rows adds
                // `row` and the next tap's weights add nt): one thread issues
                // every MMA of the CTA and must not spend more time per MMA
                // than the tensor core does.
                const uint64_t ad0 = sdesc(abase, (uint32_t)G::KC, (uint32_t)(G::AW * 16));
                const int bstep = a.flip ? -a.nt : a.nt;
                const uint64_t bd0 = sdesc(bbase, (uint32_t)B_KC, 128) + (uint64_t)(a.flip ? 26 * a.nt : 0);
                const uint32_t acc0 = tmem + (uint32_t)(buf * p.ncols);
                const uint32_t accz[TD] = {acc0, acc0 + (uint32_t)a.nt, acc0 + (uint32_t)(2 * a.nt),
                                           acc0 + (uint32_t)(3 * a.nt)};
#pragma unroll
                for (int tap = 0; tap < 27; tap++) {
                    const int kd = tap / 9, kh = (tap / 3) % 3, kw = tap % 3;
                    const uint64_t bdesc = bd0 + (uint64_t)(long long)(tap * bstep);
#pragma unroll
                    for (int zp = 0; zp < TD; zp++) {
                        const int row = ((zp + kd) * G::AH + kh) * G::AW + kw;
                        mma_bf16(accz[zp], ad0 + (uint64_t)row, bdesc, idesc, (k > 0 || tap > 0) ? 1u : 0u);
                    }
                }
                mma_commit(&empty[s]);
                if (k == nchunk - 1) mma_commit(&acc_full[buf]);
            }
            s_consumed = consumed;
            mma_commit(&done);  // arrives once every MMA issued above has completed
        }
    } else {
        const int q = warp & 3;  // the TMEM lane quarter this warp may access
        const int m = q * 32 + lane;
        for (int ti = 0; ti < my_tiles; ti++) {
            const int buf = ti & 1;
            if (!mbar_wait_ab(&acc_full[buf], (unsigned)((ti >> 1) & 1), stop, a.err)) break;
            fence_after();
            const TileAt c = tile_at(a, (int)blockIdx.x + ti * (int)gridDim.x);
            const int vw = c.w0 + (m & 7), vh = c.h0 + (m >> 3);
            const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * p.ncols);
#pragma unroll 1
            for (int zp = 0; zp < TD; zp++) {
                const int vd = c.d0 + zp;
                const bool inside = vw < a.w && vh < a.h && vd < a.d;
                const long long vox = (((long long)c.nb * a.d + vd) * a.h + vh) * a.w + vw;
#pragma unroll 1
                for (int c0 = 0; c0 < a.nt; c0 += 32) {
                    // two 16-column loads in flight before one wait (nt is 16, 32 or 64)
                    uint32_t r[2][16];
                    const int nh = a.nt - c0 >= 32 ? 2 : 1;
                    tmem_ld16_async(lane_addr + (uint32_t)(zp * a.nt + c0), r[0]);
                    if (nh == 2) tmem_ld16_async(lane_addr + (uint32_t)(zp * a.nt + c0 + 16), r[1]);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (!inside) continue;
#pragma unroll
                    for (int hh = 0; hh < 2; hh++) {
                        if (hh >= nh) break;
                        const int ch = c.n0 + c0 + hh * 16;
                        float v[16];
#pragma unroll
                        for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[hh][j]);
                        if (a.bias) {
#pragma unroll
                            for (int j = 0; j < 16; j++) v[j] += a.bias[ch + j];
                        }
                        if (a.relu) {
#pragma unroll
                            for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j], 0.f);
                        }
                        if (a.mask) {
                            const uint4* mp = reinterpret_cast<const uint4*>(a.mask + vox * a.ms + a.mo + ch);
                            uint4 mv[2] = {mp[0], mp[1]};
                            const unsigned short* mb = reinterpret_cast<const unsigned short*>(mv);
#pragma unroll
                            for (int j = 0; j < 16; j++)
                                if (!bf16_pos(mb[j])) v[j] = 0.f;
                        }
                        __align__(16) __nv_bfloat162 o[8];
#pragma unroll
                        for (int j = 0; j < 8; j++) o[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                        uint4* dst = reinterpret_cast<uint4*>(a.y + vox * a.ys + a.yo + ch);
                        dst[0] = reinterpret_cast<const uint4*>(o)[0];
                        dst[1] = reinterpret_cast<const uint4*>(o)[1];
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[buf]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 32 && !mbar_wait(&done, 0)) atomicOr(a.err, 2u);
    if (threadIdx.x == 0 && s_stop) {
        // let the copies still in flight land before the CTA's shared memory goes away
        for (int j = s_consumed; j < s_issued; j++) mbar_wait(&full[j % S], (unsigned)((j / S) & 1));
        if (p.wres) mbar_wait(&wfull, 0);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, 2 * p.ncols);
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
constexpr int WG_MAX_MT = 8;

struct WgArgs {
    const __nv_bfloat16* x;  // input activation [vox][cin]
    const __nv_bfloat16* g;  // gradient of the pre-activation output [vox][cout]
    int taps, cin, cout;
    int n, d, h, w;
    int rows;                // taps * cin
    int mt;                  // 128-row tiles per CTA
    int groups;
    long long vox;           // voxels
    long long steps;         // ceil(voxels / 16); the ragged last step is zero-padded
    int ksplit;
    float* dw;               // [taps][cout][cin], accumulated
    unsigned* err;
};

__global__ void __launch_bounds__(CONV_THREADS) k_conv_wgrad(const WgArgs a) {
    extern __shared__ __align__(128) unsigned char smraw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smraw + 127) & ~(uintptr_t)127);
    __shared__ __align__(8) uint64_t bar[2], done;
    __shared__ uint32_t tmem_base;

    const int grp = blockIdx.x % a.groups;
    const int ks = blockIdx.x / a.groups;
    const int R = a.mt * 128;  // rows staged per step
    const int row0 = grp * R;
    const int A_KC = R * 16;
    const int B_KC = a.cout * 16;
    const int stage_bytes = 2 * A_KC + 2 * B_KC;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ncols = tmem_cols(a.mt * a.cout);
    const long long s_begin = a.steps * ks / a.ksplit, s_end = a.steps * (ks + 1) / a.ksplit;

    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(&tmem_base, ncols);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = idesc_bf16(a.cout);
    const int k = threadIdx.x & 15;  // this thread's voxel within each step
    const long long plane = (long long)a.h * a.w;
    bool ok = true;

    for (long long s = s_begin; s < s_end; s++) {
        const int it = (int)(s - s_begin);
        const int st = it & 1;
        // the MMAs that read this stage two steps ago must be done
        if (it >= 2 && !mbar_wait(&bar[st], (unsigned)(((it - 2) >> 1) & 1))) ok = false;
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        unsigned char* A = sm + st * stage_bytes;
        unsigned char* Bm = A + 2 * A_KC;
        const long long v = s * 16 + k;
        const bool live = v < a.vox;
        const int vw = (int)(v % a.w), vh = (int)((v / a.w) % a.h), vd = (int)((v / plane) % a.d);
        const int kc = k >> 3, kk = k & 7;
        // A: rows (tap, c) of this group, column k
        for (int u = threadIdx.x >> 4; u < R / 8; u += CONV_THREADS / 16) {
            const int r = row0 + u * 8;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (live && r < a.rows) {
                const int tap = r / a.cin, c = r % a.cin;
                int dd = 0, dh = 0, dw = 0;
                if (a.taps == 27) {
                    dd = tap / 9 - 1;
                    dh = (tap / 3) % 3 - 1;
                    dw = tap % 3 - 1;
                }
                const int sw = vw + dw, sh = vh + dh, sd = vd + dd;
                if (sw >= 0 && sw < a.w && sh >= 0 && sh < a.h && sd >= 0 && sd < a.d) {
                    const long long sv = v + ((long long)dd * a.h + dh) * a.w + dw;
                    val = *reinterpret_cast<const uint4*>(a.x + sv * a.cin + c);
                }
            }
            const unsigned short* e = reinterpret_cast<const unsigned short*>(&val);
            unsigned short* base = reinterpret_cast<unsigned short*>(A + kc * A_KC + (u * 8) * 16) + kk;
#pragma unroll
            for (int j = 0; j < 8; j++) base[j * 8] = e[j];
        }
        // B: rows n, column k
        for (int u = threadIdx.x >> 4; u < a.cout / 8; u += CONV_THREADS / 16) {
            const uint4 val = live ? *reinterpret_cast<const uint4*>(a.g + v * a.cout + u * 8) : make_uint4(0, 0, 0, 0);
            const unsigned short* e = reinterpret_cast<const unsigned short*>(&val);
            unsigned short* base = reinterpret_cast<unsigned short*>(Bm + kc * B_KC + (u * 8) * 16) + kk;
#pragma unroll
            for (int j = 0; j < 8; j++) base[j * 8] = e[j];
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            fence_after();
            const uint64_t bdesc = sdesc(s32(Bm), (uint32_t)B_KC, 128);
            for (int mt = 0; mt < a.mt; mt++) {
                const uint64_t adesc = sdesc(s32(A + mt * 128 * 16), (uint32_t)A_KC, 128);
                mma_bf16(tmem + (uint32_t)(mt * a.cout), adesc, bdesc, idesc, it > 0 ? 1u : 0u);
            }
            mma_commit(&bar[st]);
        }
    }
    if (threadIdx.x == 0) mma_commit(&done);
    __syncthreads();
    const bool fin = mbar_wait(&done, 0);
    if (__syncthreads_or(!fin || !ok)) {
        if (threadIdx.x == 0) atomicOr(a.err, 4u);
    } else if (s_end > s_begin) {
        fence_after();
        for (int mt = 0; mt < a.mt; mt++) {
            const int r = row0 + mt * 128 + warp * 32 + lane;
            const int tap = r / a.cin, c = r % a.cin;
            for (int n0 = 0; n0 < a.cout; n0 += 16) {
                uint32_t v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mt * a.cout + n0), v);
                if (r < a.rows) {
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        atomicAdd(a.dw + ((long long)tap * a.cout + n0 + j) * a.cin + c, __uint_as_float(v[j]));
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, ncols);
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int pick_nt(int cout, int ntmax) {
    if (cout <= ntmax) return cout;
    for (int nt = ntmax; nt >= 16; nt -= 16)
        if (cout % nt == 0) return nt;
    return 16;
}

}  // namespace

// activations [n][d][h][w][c] bf16 read in halo boxes of 8 channels
bool conv_act_map(CUtensorMap* m, const void* base, int n, int d, int h, int w, int c, int taps) {
    auto enc = encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(base) & 15) || c % 16) return false;
    const int H = taps == 27 ? 1 : 0;
    cuuint64_t dims[5] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)d, (cuuint64_t)n};
    cuuint64_t str[4] = {(cuuint64_t)c * 2, (cuuint64_t)c * 2 * w, (cuuint64_t)c * 2 * w * h,
                         (cuuint64_t)c * 2 * w * h * d};
    cuuint32_t box[5] = {8, (cuuint32_t)(TW + 2 * H), (cuuint32_t)(TH + 2 * H), (cuuint32_t)(TD + 2 * H), 1};
    cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, str, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// weights [taps][rows][kdim] bf16 read as (8 of kdim) x nt rows x all taps
bool conv_wt_map(CUtensorMap* m, const void* base, int taps, int rows, int kdim, int nt) {
    auto enc = encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(base) & 15) || kdim % 16) return false;
    cuuint64_t dims[3] = {(cuuint64_t)kdim, (cuuint64_t)rows, (cuuint64_t)taps};
    cuuint64_t str[2] = {(cuuint64_t)kdim * 2, (cuuint64_t)kdim * 2 * rows};
    cuuint32_t box[3] = {8, (cuuint32_t)nt, (cuuint32_t)taps};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, str, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int conv_nt(int taps, int cout) { return pick_nt(cout, taps == 27 ? 64 : 128); }

int launch_conv_mma(const ConvLaunch& L, cudaStream_t s) {
    const int taps = L.taps;
    if ((taps != 27 && taps != 1) || L.cin % 16 || L.cout % 16 || L.cin <= 0 || L.cout <= 0) return FSIM_E_INVALID;
    if (L.ys % 8 || L.yo % 8 || (L.mask && (L.ms % 8 || L.mo % 8))) return FSIM_E_INVALID;
    MmaArgs a{};
    a.n = L.n; a.d = L.d; a.h = L.h; a.w = L.w;
    a.cin = L.cin; a.cout = L.cout;
    a.nt = conv_nt(taps, L.cout);
    a.tiles_w = ceil_div(L.w, TW);
    a.tiles_h = ceil_div(L.h, TH);
    a.tiles_d = ceil_div(L.d, TD);
    a.ntiles = L.cout / a.nt;
    a.flip = L.flip;
    a.bias = L.bias;
    a.relu = L.relu;
    a.mask = L.mask; a.ms = L.ms; a.mo = L.mo;
    a.y = L.y; a.ys = L.ys; a.yo = L.yo;
    a.err = L.err;
    const long long grid = (long long)a.tiles_w * a.tiles_h * a.tiles_d * L.n * a.ntiles;
    if (grid <= 0) return FSIM_OK;
    const int nchunk = L.cin / 16;
    if (taps == 27) {
        if (grid >= (1ll << 31)) return FSIM_E_INVALID;
        PersArgs p{};
        const int A = Halo<27>::A_BYTES, B_KC = 27 * a.nt * 16, w_all = nchunk * 2 * B_KC;
        p.total_tiles = (int)grid;
        p.ncols = tmem_cols(TD * a.nt);
        if (2 * p.ncols > 512) return FSIM_E_INVALID;
        const int room = SMEM_LIMIT - 128;
        if (a.ntiles == 1 && w_all + 2 * A <= room) {
            p.wres = 1;
            p.stage_bytes = A;
            a.stages = (room - w_all) / A;
        } else {
            p.wres = 0;
            p.stage_bytes = A + 2 * B_KC;
            a.stages = room / p.stage_bytes;
        }
        if (a.stages < 2) return FSIM_E_INVALID;
        if (a.stages > PERS_MAX_STAGES) a.stages = PERS_MAX_STAGES;
        p.m = a;
        int smem = a.stages * p.stage_bytes + (p.wres ? w_all : 0) + 128;
        if (smem < SMEM_LIMIT / 2 + 1024) smem = SMEM_LIMIT / 2 + 1024;  // one CTA per SM
        static int sms[64] = {0};
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FSIM_E_CUDA;
        if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return FSIM_E_CUDA;
        const int ctas = grid < sms[dev] ? (int)grid : sms[dev];
        if (set_smem_limit((const void*)k_conv_pers, SMEM_LIMIT) != cudaSuccess) return FSIM_E_CUDA;
        k_conv_pers<<<ctas, PERS_THREADS, smem, s>>>(p, *L.mx, *L.mw);
        return cudaGetLastError() == cudaSuccess ? FSIM_OK : FSIM_E_CUDA;
    }
    const int a_bytes = Halo<1>::A_BYTES;
    const int stage = a_bytes + 2 * a.nt * 16;
    if (stage + 128 > SMEM_LIMIT) return FSIM_E_INVALID;
    // as many pipeline stages (<= 3, <= chunks) as keep two CTAs on an SM: the
    // second CTA's loads and epilogue overlap the first one's MMAs
    int stages = 1;
    while (stages < 3 && stages < nchunk && (stages + 1) * stage + 128 <= SMEM_LIMIT / 2) stages++;
    a.stages = stages;
    int smem = stages * stage + 128;
    // the pointwise kernel's accumulator can take all of TMEM: one CTA per SM
    if (smem < 160 * 1024) smem = 160 * 1024;
    if (set_smem_limit((const void*)k_conv_mma<1>, SMEM_LIMIT) != cudaSuccess) return FSIM_E_CUDA;
    k_conv_mma<1><<<(unsigned)grid, CONV_THREADS, smem, s>>>(a, *L.mx, *L.mw);
    return cudaGetLastError() == cudaSuccess ? FSIM_OK : FSIM_E_CUDA;
}

int launch_conv_wgrad(const WgradLaunch& L, cudaStream_t s) {
    if ((L.taps != 27 && L.taps != 1) || L.cin % 16 || L.cout % 16 || L.cout > 64) return FSIM_E_INVALID;
    const long long vox = (long long)L.n * L.d * L.h * L.w;
    if (vox <= 0) return FSIM_OK;
    WgArgs a{};
    a.x = L.x; a.g = L.g;
    a.taps = L.taps; a.cin = L.cin; a.cout = L.cout;
    a.n = L.n; a.d = L.d; a.h = L.h; a.w = L.w;
    a.rows = L.taps * L.cin;
    const int tiles = ceil_div(a.rows, 128);
    int mt = 512 / tmem_cols(L.cout);
    if (mt > WG_MAX_MT) mt = WG_MAX_MT;
    if (mt > tiles) mt = tiles;
    while (mt > 1 && tmem_cols(mt * L.cout) > 512) mt--;
    a.mt = mt;
    a.groups = ceil_div(tiles, mt);
    a.vox = vox;
    a.steps = (vox + 15) / 16;
    int ks = (int)((4LL * 152 + a.groups - 1) / a.groups);
    const long long max_ks = a.steps / 8 > 0 ? a.steps / 8 : 1;
    if (ks > max_ks) ks = (int)max_ks;
    if (ks < 1) ks = 1;
    a.ksplit = ks;
    a.dw = L.dw;
    a.err = L.err;
    const int stage = 2 * (mt * 128 * 16) + 2 * L.cout * 16;
    const int smem = 2 * stage + 128;
    if (set_smem_limit((const void*)k_conv_wgrad, SMEM_LIMIT) != cudaSuccess) return FSIM_E_CUDA;
    k_conv_wgrad<<<(unsigned)(a.groups * a.ksplit), CONV_THREADS, smem, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? FSIM_OK : FSIM_E_CUDA;
}
