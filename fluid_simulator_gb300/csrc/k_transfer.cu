// k_transfer.cu -- particle <-> grid transfers on cell-sorted particles.
//
// Both kernels work on tiles of TX x TY x TZ cells (one CTA per tile).
//
// P2G (Simulator::p2gTransfer, simulator.cpp:314-352, fused with
// markFluidCellsAndCalculateParticleDensities, simulator.cpp:354-368): the CTA
// owns the faces and cell centres of its tile and computes their final values,
// so no grid accumulator ever goes to global memory and no global atomic is
// used.  Each thread takes one cell of the tile plus its one-cell halo, walks
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

#include "fsim_ctx.h"

namespace {

constexpr int TX = 8, TY = 8, TZ = 32;
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
constexpr int TCELLS = TX * TY * TZ;
constexpr int P2G_THREADS = 256;
constexpr int P2G_SMEM = 7 * TCELLS * (int)sizeof(float);

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

template <bool APIC>
__global__ void __launch_bounds__(P2G_THREADS) k_p2g(const P2GArgs a) {
    extern __shared__ float sm[];
    float* s_vw = sm;              // [3][TCELLS] sum of w * contribution
    float* s_w = sm + 3 * TCELLS;  // [3][TCELLS] sum of w
    float* s_avg = sm + 6 * TCELLS;
    for (int k = threadIdx.x; k < 7 * TCELLS; k += blockDim.x) sm[k] = 0.f;
    const int bt = blockIdx.x;
    const int tz = bt % a.ntz, ty = (bt / a.ntz) % a.nty, tx = bt / (a.ntz * a.nty);
    const int x0 = tx * TX, y0 = ty * TY, z0 = tz * TZ;
    __syncthreads();
    const float hinv = a.g.hinv, h = a.g.h;

    for (int hc = threadIdx.x; hc < HX * HY * HZ; hc += blockDim.x) {
        const int hz = hc % HZ, hy = (hc / HZ) % HY, hx = hc / (HZ * HY);
        const int cx = x0 - 1 + hx, cy = y0 - 1 + hy, cz = z0 - 1 + hz;
        if (cx < 0 || cy < 0 || cz < 0 || cx >= a.g.nx || cy >= a.g.ny || cz >= a.g.nz) continue;
        const long long cell = gidx(a.g, cx, cy, cz);
        const int beg = a.cstart[cell], end = a.cstart[cell + 1];
        for (int k = beg; k < end; k++) {
            const uint32_t i = a.perm[k];
            const float g[3] = {a.p.p[0][i] * hinv, a.p.p[1][i] * hinv, a.p.p[2][i] * hinv};
            const float vv[3] = {a.p.v[0][i], a.p.v[1][i], a.p.v[2][i]};
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
                float cvec[3] = {0.f, 0.f, 0.f};
                if (APIC) {
                    cvec[0] = a.p.c[3 * ax][i];
                    cvec[1] = a.p.c[3 * ax + 1][i];
                    cvec[2] = a.p.c[3 * ax + 2][i];
                }
                // stencil of MacGrid::getFacesAround (macGrid.cpp:142-181)
                int b[3];
                float d0[3];
#pragma unroll
                for (int dd = 0; dd < 3; dd++) {
                    const float off = (dd == ax) ? 0.f : 0.5f;
                    b[dd] = (int)(g[dd] - off) - (dd == ax ? 1 : 0);
                    // node of cell t for this face axis: t + 1 along ax, t + 0.5 across
                    d0[dd] = g[dd] - ((float)b[dd] + (dd == ax ? 1.f : 0.5f));
                }
                const float w0[3] = {1.f - fabsf(d0[0]), 1.f - fabsf(d0[1]), 1.f - fabsf(d0[2])};
                const float w1[3] = {1.f - fabsf(d0[0] - 1.f), 1.f - fabsf(d0[1] - 1.f),
                                     1.f - fabsf(d0[2] - 1.f)};
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
                    const int lx = b[0] + ox - x0, ly = b[1] + oy - y0, lz = b[2] + oz - z0;
                    if (lx < 0 || ly < 0 || lz < 0 || lx >= TX || ly >= TY || lz >= TZ) continue;
                    const float w = (ox ? w1[0] : w0[0]) * (oy ? w1[1] : w0[1]) * (oz ? w1[2] : w0[2]);
                    float contrib = vv[ax];
                    if (APIC) {
                        // c[ax] . (face.pos - pos) with face.pos - pos = -(g - node) * h
                        const float ddx = d0[0] - (float)ox, ddy = d0[1] - (float)oy, ddz = d0[2] - (float)oz;
                        contrib -= (cvec[0] * ddx + cvec[1] * ddy + cvec[2] * ddz) * h;
                    }
                    const int li = (lx * TY + ly) * TZ + lz;
                    atomicAdd(&s_vw[ax * TCELLS + li], contrib * w);
                    atomicAdd(&s_w[ax * TCELLS + li], w);
                }
            }
            // cell-centre density (MacGrid::getCellsAround, macGrid.cpp:188-202)
            {
                int b[3];
                float d0[3];
#pragma unroll
                for (int dd = 0; dd < 3; dd++) {
                    b[dd] = (int)(g[dd] - 0.5f);
                    d0[dd] = g[dd] - ((float)b[dd] + 0.5f);
                }
#pragma unroll
                for (int o = 0; o < 8; o++) {
                    const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
                    const int lx = b[0] + ox - x0, ly = b[1] + oy - y0, lz = b[2] + oz - z0;
                    if (lx < 0 || ly < 0 || lz < 0 || lx >= TX || ly >= TY || lz >= TZ) continue;
                    const float w = (1.f - fabsf(d0[0] - ox)) * (1.f - fabsf(d0[1] - oy)) *
                                    (1.f - fabsf(d0[2] - oz));
                    atomicAdd(&s_avg[(lx * TY + ly) * TZ + lz], w);
                }
            }
        }
    }
    __syncthreads();
    for (int lc = threadIdx.x; lc < TCELLS; lc += blockDim.x) {
        const int lz = lc % TZ, ly = (lc / TZ) % TY, lx = lc / (TZ * TY);
        const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
        if (x >= a.g.nx || y >= a.g.ny || z >= a.g.nz) continue;
        const long long cell = gidx(a.g, x, y, z);
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            const float w = s_w[ax * TCELLS + lc];
            a.u[ax][cell] = (w > 1e-6f) ? s_vw[ax * TCELLS + lc] / w : 0.f;
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
    // wait for the staged grid (bounded: about 2^31 cycles, then report and leave;
    // the leave decision is made for the whole CTA at once)
    {
        const long long t0 = clock64();
        bool ok = false;
        while (!(ok = mbar_try_wait(&mbar, 0))) {
            if (clock64() - t0 > (1ll << 31)) break;
        }
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicOr(a.err, FSIM_DERR_TMA_TIMEOUT);
            return;
        }
    }
    const int total = seg_pre[TX * TY];
    const float hinv = a.g.hinv;
    for (int j = threadIdx.x; j < total; j += blockDim.x) {
        int lo = 0, hi = TX * TY - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (seg_pre[mid] <= j) lo = mid; else hi = mid - 1;
        }
        const int k = seg_beg[lo] + (j - seg_pre[lo]);
        const uint32_t i = a.perm[k];
        const float px = a.src.p[0][i], py = a.src.p[1][i], pz = a.src.p[2][i];
        const float g[3] = {px * hinv, py * hinv, pz * hinv};
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
            float pic = 0.f, flip = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
            for (int o = 0; o < 8; o++) {
                const int ox = o >> 2, oy = (o >> 1) & 1, oz = o & 1;
                const float dx = d0[0] - ox, dy = d0[1] - oy, dz = d0[2] - oz;
                const float wx = 1.f - fabsf(dx), wy = 1.f - fabsf(dy), wz = 1.f - fabsf(dz);
                const float w = wx * wy * wz;
                const int si = ((sx + ox) * BY + (sy + oy)) * BZ + (sz + oz);
                const float v2 = sv2[ax * BOXN + si];
                pic += v2 * w;
                if (MODE == 1) flip += (v2 - su[ax * BOXN + si]) * w;
                if (MODE == 2) {
                    // trilinearInterpollGradient (util/interpolation.h:21-35)
                    const float gx = (dx > 0.f ? -1.f : 1.f) * wy * wz * hinv;
                    const float gy = (dy > 0.f ? -1.f : 1.f) * wx * wz * hinv;
                    const float gz = (dz > 0.f ? -1.f : 1.f) * wx * wy * hinv;
                    c0 += gx * v2;
                    c1 += gy * v2;
                    c2 += gz * v2;
                }
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

void launch_p2g(fsim_ctx* ctx) {
    const GridGeom& g = ctx->g;
    P2GArgs a;
    a.p = ctx->buf[ctx->cur];
    a.perm = ctx->perm;
    a.cstart = ctx->cstart;
    a.g = g;
    for (int k = 0; k < 3; k++) a.u[k] = ctx->u[k];
    a.flags = ctx->flags;
    a.avg = ctx->avg;
    a.ntx = ceil_div(g.nx, TX);
    a.nty = ceil_div(g.ny, TY);
    a.ntz = ceil_div(g.nz, TZ);
    const int nb = a.ntx * a.nty * a.ntz;
    ctx->launches += 1;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_p2g<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, P2G_SMEM);
        cudaFuncSetAttribute(k_p2g<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, P2G_SMEM);
        attr_set = true;
    }
    if (ctx->prm.transfer == FSIM_APIC)
        k_p2g<true><<<nb, P2G_THREADS, P2G_SMEM, ctx->stream>>>(a);
    else
        k_p2g<false><<<nb, P2G_THREADS, P2G_SMEM, ctx->stream>>>(a);
}

// P2G on caller-provided buffers (used by the allocation-free entry point in
// fsim_static.cu); same kernel as launch_p2g.
void launch_p2g_raw(ParticleBuf p, const uint32_t* perm, const int* cstart, const GridGeom& g, float* const u[3],
                    uint8_t* flags, float* avg, bool apic, cudaStream_t stream) {
    P2GArgs a;
    a.p = p;
    a.perm = perm;
    a.cstart = cstart;
    a.g = g;
    for (int k = 0; k < 3; k++) a.u[k] = u[k];
    a.flags = flags;
    a.avg = avg;
    a.ntx = ceil_div(g.nx, TX);
    a.nty = ceil_div(g.ny, TY);
    a.ntz = ceil_div(g.nz, TZ);
    const int nb = a.ntx * a.nty * a.ntz;
    cudaFuncSetAttribute(k_p2g<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, P2G_SMEM);
    cudaFuncSetAttribute(k_p2g<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, P2G_SMEM);
    if (apic)
        k_p2g<true><<<nb, P2G_THREADS, P2G_SMEM, stream>>>(a);
    else
        k_p2g<false><<<nb, P2G_THREADS, P2G_SMEM, stream>>>(a);
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
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_g2p<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * BOXN * 4);
        cudaFuncSetAttribute(k_g2p<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 6 * BOXN * 4);
        cudaFuncSetAttribute(k_g2p<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * BOXN * 4);
        attr_set = true;
    }
    const CUtensorMap* m = ctx->tmap;
    if (mode == FSIM_PIC)
        k_g2p<0><<<nb, G2P_THREADS, smem, ctx->stream>>>(a, m[0], m[1], m[2], m[3], m[4], m[5]);
    else if (mode == FSIM_FLIP)
        k_g2p<1><<<nb, G2P_THREADS, smem, ctx->stream>>>(a, m[0], m[1], m[2], m[3], m[4], m[5]);
    else
        k_g2p<2><<<nb, G2P_THREADS, smem, ctx->stream>>>(a, m[0], m[1], m[2], m[3], m[4], m[5]);
    return 0;
}
