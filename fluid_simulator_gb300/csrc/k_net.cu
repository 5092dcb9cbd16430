// k_net.cu -- the pressure warm-start network: data-movement kernels (input
// packing, space-to-depth, trilinear up-sampling and their adjoints), the
// head and loss, bias gradients, Adam, weight packing, and the host-side
// forward / backward / training step / solver hook.  The convolutions run on
// the tensor cores (k_conv.cu).
//
// The network has no counterpart in the reference, whose PCG always starts
// from zero pressure (src/Simulator/simulator/macGrid/bridsonSolverGrid.cpp:249).
// Its output is only an initial guess: the solver judges it against the
// previous step's pressure by residual and still iterates to its tolerance.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fsim_ctx.h"
#include "fsim_net.h"

namespace {

using bf16 = __nv_bfloat16;
constexpr int NT_THREADS = 256;
constexpr uint16_t CODE_FLUID_BIT = 0x8000;

__device__ __forceinline__ void ld8(const bf16* p, float (&v)[8]) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float2 f = __bfloat1622float2(h[j]);
        v[2 * j] = f.x;
        v[2 * j + 1] = f.y;
    }
}
__device__ __forceinline__ void st8(bf16* p, const float (&v)[8]) {
    uint4 u;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
    for (int j = 0; j < 4; j++) h[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
    *reinterpret_cast<uint4*>(p) = u;
}

// ---- input ----------------------------------------------------------------
// in: [vox][4] FP32 (rhs scaled, fluid, solid, air) -> x0: [vox][16] bf16
__global__ void k_pack_input(const float* in, long long vox, bf16* x0) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vox) return;
    const float4 q = *reinterpret_cast<const float4*>(in + v * 4);
    const float a[8] = {q.x, q.y, q.z, q.w, 0.f, 0.f, 0.f, 0.f};
    const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    st8(x0 + v * 16, a);
    st8(x0 + v * 16 + 8, z);
}

__global__ void k_to_bf16(const float* in, long long n, bf16* out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}
__global__ void k_to_f32(const bf16* in, long long n, float* out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __bfloat162float(in[i]);
}

// ---- space-to-depth (2x2x2 stride-2 down-convolution = s2d + pointwise) -----
// dst[coarse][(sd*4 + sh*2 + sw)*C + c] = src[2*coarse + (sd, sh, sw)][c]
__global__ void k_s2d(const bf16* src, int ss, int so, int C, int n, int D, int H, int W, bf16* dst) {
    const int oct = C / 8;
    const long long total = (long long)n * (D / 2) * (H / 2) * (W / 2) * 8 * oct;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int o = (int)(i % oct);
    long long t = i / oct;
    const int sub = (int)(t % 8);
    const long long cv = t / 8;  // coarse voxel
    const int cw = (int)(cv % (W / 2)), chh = (int)((cv / (W / 2)) % (H / 2));
    const long long cdn = cv / ((long long)(W / 2) * (H / 2));  // n * D/2 + cd
    const int cd = (int)(cdn % (D / 2));
    const int nb = (int)(cdn / (D / 2));
    const int fd = 2 * cd + (sub >> 2), fh = 2 * chh + ((sub >> 1) & 1), fw = 2 * cw + (sub & 1);
    const long long fv = (((long long)nb * D + fd) * H + fh) * W + fw;
    *reinterpret_cast<uint4*>(dst + cv * 8 * C + sub * C + o * 8) =
        *reinterpret_cast<const uint4*>(src + fv * ss + so + o * 8);
}

// out[fine][c] = (gs[coarse][sub*C + c] + gc[fine][gco + c]) * (m[fine][mo + c] > 0)
__global__ void k_d2s_add_mask(const bf16* gs, const bf16* gc, int gcs, int gco, const bf16* m, int ms, int mo,
                               int C, int n, int D, int H, int W, bf16* out) {
    const int oct = C / 8;
    const long long total = (long long)n * D * H * W * oct;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int o = (int)(i % oct);
    const long long fv = i / oct;
    const int fw = (int)(fv % W), fh = (int)((fv / W) % H);
    const long long fdn = fv / ((long long)W * H);
    const int fd = (int)(fdn % D), nb = (int)(fdn / D);
    const long long cv = (((long long)nb * (D / 2) + fd / 2) * (H / 2) + fh / 2) * (W / 2) + fw / 2;
    const int sub = ((fd & 1) << 2) | ((fh & 1) << 1) | (fw & 1);
    float a[8], b[8], mk[8];
    ld8(gs + cv * 8 * C + sub * C + o * 8, a);
    ld8(gc + fv * gcs + gco + o * 8, b);
    ld8(m + fv * ms + mo + o * 8, mk);
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = mk[j] > 0.f ? a[j] + b[j] : 0.f;
    st8(out + fv * C + o * 8, a);
}

// ---- trilinear 2x up-sampling (align_corners = false) -------------------------
__device__ __forceinline__ void up_src(int f, int nc, int& i0, int& i1, float& l1) {
    float s = (f + 0.5f) * 0.5f - 0.5f;
    if (s < 0.f) s = 0.f;
    i0 = (int)s;
    i1 = i0 < nc - 1 ? i0 + 1 : i0;
    l1 = s - (float)i0;
}

// src: coarse [n][D][H][W][C]; dst: fine, channel stride ds (offset 0).
// One thread per (coarse voxel, 8-channel octet) writes the 2x2x2 fine voxels
// whose lower trilinear corner lies at or next to it: fine 2k reads coarse
// k-1 and k, fine 2k+1 reads k and k+1 (clamped at the border).  Per fine
// (d, h) pair the thread reads the 2 x 2 coarse rows at k-1 and k, writes fine
// w = 2k, then reads the rows at k+1 and writes w = 2k+1, sharing the samples
// at k.  The weights and the summation order are those of the per-voxel
// formula (corner k = (d, h, w) bits, weight = product of the three 1-D
// weights), so the result does not depend on this blocking.  Coarse indices
// are 32-bit: the host keeps n * D * H * W * (C / 8) below 2^31.
__device__ __forceinline__ void up_out(const uint4 (&lo)[4], const uint4 (&hi)[4], bool w0_hi, bool w1_hi, float ld,
                                       float lh, float lw, bf16* out) {
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float wt = ((k & 4) ? ld : 1.f - ld) * ((k & 2) ? lh : 1.f - lh) * ((k & 1) ? lw : 1.f - lw);
        const int r = ((k & 4) ? 2 : 0) | ((k & 2) ? 1 : 0);
        const bool use_hi = (k & 1) ? w1_hi : w0_hi;
        const uint4 u = use_hi ? hi[r] : lo[r];
        const __nv_bfloat162* hv = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float2 f = __bfloat1622float2(hv[j]);
            acc[2 * j] += wt * f.x;
            acc[2 * j + 1] += wt * f.y;
        }
    }
    st8(out, acc);
}

__global__ void __launch_bounds__(NT_THREADS, 3) k_upsample(const bf16* src, int C, int n, int D, int H, int W,
                                                            bf16* dst, int ds) {
    const int oct = C >> 3;
    const int total = n * D * H * W * oct;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int o = i % oct;
    int t = i / oct;
    const int cw = t % W;
    t /= W;
    const int chh = t % H;
    t /= H;
    const int cd = t % D;
    const int nb = t / D;
    const int FD = 2 * D, FH = 2 * H, FW = 2 * W;
    const int wl = cw > 0 ? cw - 1 : 0, wr = cw < W - 1 ? cw + 1 : cw;
    // fine w = 2cw reads coarse {i0, i1} in {wl, cw}; fine 2cw + 1 reads them in {cw, wr}
    int a0, a1, b0, b1;
    float lwa, lwb;
    up_src(2 * cw, W, a0, a1, lwa);
    up_src(2 * cw + 1, W, b0, b1, lwb);
#pragma unroll 1
    for (int a = 0; a < 2; a++) {
        int d0, d1;
        float ld;
        up_src(2 * cd + a, D, d0, d1, ld);
#pragma unroll 1
        for (int b = 0; b < 2; b++) {
            int h0, h1;
            float lh;
            up_src(2 * chh + b, H, h0, h1, lh);
            size_t rowb[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int dd = (r & 2) ? d1 : d0, hh = (r & 1) ? h1 : h0;
                rowb[r] = ((size_t)((nb * D + dd) * H + hh) * W) * C + o * 8;
            }
            uint4 lo[4], mid[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                lo[r] = *reinterpret_cast<const uint4*>(src + rowb[r] + (size_t)wl * C);
                mid[r] = *reinterpret_cast<const uint4*>(src + rowb[r] + (size_t)cw * C);
            }
            const size_t fv = ((size_t)(nb * FD + 2 * cd + a) * FH + 2 * chh + b) * FW + 2 * cw;
            up_out(lo, mid, a0 != wl, a1 != wl, ld, lh, lwa, dst + fv * ds + o * 8);
#pragma unroll
            for (int r = 0; r < 4; r++) lo[r] = *reinterpret_cast<const uint4*>(src + rowb[r] + (size_t)wr * C);
            up_out(mid, lo, b0 != cw, b1 != cw, ld, lh, lwb, dst + (fv + 1) * ds + o * 8);
        }
    }
}

// weights of coarse index k in the fine samples near it (adjoint of up_src)
__device__ __forceinline__ int up_adj(int k, int nc, int (&f)[6], float (&w)[6]) {
    int cnt = 0;
    for (int ff = 2 * k - 2; ff <= 2 * k + 3; ff++) {
        if (ff < 0 || ff >= 2 * nc) continue;
        int i0, i1;
        float l1;
        up_src(ff, nc, i0, i1, l1);
        float wt = 0.f;
        if (i0 == k) wt += 1.f - l1;
        if (i1 == k) wt += l1;
        if (wt != 0.f) {
            f[cnt] = ff;
            w[cnt] = wt;
            cnt++;
        }
    }
    return cnt;
}

// out[coarse][c] = (sum_fine w * g[fine][c]) * (m[coarse][c] > 0); g channel stride gs (offset 0)
__global__ void k_upsample_bwd(const bf16* g, int gs, const bf16* m, int C, int n, int D, int H, int W, bf16* out) {
    const int oct = C / 8;
    const long long total = (long long)n * D * H * W * oct;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int o = (int)(i % oct);
    const long long cv = i / oct;
    const int cw = (int)(cv % W), chh = (int)((cv / W) % H);
    const long long cdn = cv / ((long long)W * H);
    const int cd = (int)(cdn % D), nb = (int)(cdn / D);
    int fd[6], fh[6], fw[6];
    float wd[6], wh[6], ww[6];
    const int nd = up_adj(cd, D, fd, wd), nh = up_adj(chh, H, fh, wh), nw = up_adj(cw, W, fw, ww);
    const int FD = 2 * D, FH = 2 * H, FW = 2 * W;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int a = 0; a < nd; a++)
        for (int b = 0; b < nh; b++)
            for (int c = 0; c < nw; c++) {
                const float wt = wd[a] * wh[b] * ww[c];
                float v[8];
                ld8(g + ((((long long)nb * FD + fd[a]) * FH + fh[b]) * FW + fw[c]) * gs + o * 8, v);
#pragma unroll
                for (int j = 0; j < 8; j++) acc[j] += wt * v[j];
            }
    float mk[8];
    ld8(m + cv * C + o * 8, mk);
#pragma unroll
    for (int j = 0; j < 8; j++)
        if (!(mk[j] > 0.f)) acc[j] = 0.f;
    st8(out + cv * C + o * 8, acc);
}

// ---- head (1x1x1, 16 -> 1) and loss ---------------------------------------
__global__ void k_head(const bf16* d0, long long vox, const float* wgt, const float* bias, float scale, float* out) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vox) return;
    float a[8], b[8];
    ld8(d0 + v * 16, a);
    ld8(d0 + v * 16 + 8, b);
    float s = bias[0];
#pragma unroll
    for (int j = 0; j < 8; j++) s += a[j] * wgt[j] + b[j] * wgt[8 + j];
    out[v] = scale * s;
}

// ---- loss: relative residual of the guess + weighted relative L2 error -------
// Per sample s of the batch, with e = out - target on the fluid voxels (mask),
// A the solver's 7-point operator of the sample's cell types (diagonal: the
// non-solid neighbours; -1 per fluid neighbour; voxels outside the volume
// count as solid) and b the scaled rhs (input channel 0): since A target = b,
// r = A e is the residual b - A out the guess leaves in PCG, and
//   L_s = ||r|| / ||b|| + lam ||e|| / ||target||,   loss = mean_s L_s.
// Pass 1 stores r and adds the per-sample sums of r^2, e^2, target^2, b^2;
// k_loss_coef turns them into the loss and the per-sample gradient factors;
// pass 2 writes dloss/dout = c_r A r + c_e e.  Warps never straddle two
// samples (each sample's voxel count is a multiple of 512).
__device__ __forceinline__ bool vox_solid(const bf16* x0, long long v) { return __bfloat162float(x0[v * 16 + 2]) > 0.5f; }

template <bool GRAD>
__global__ void k_loss(const float* out, const float* target, const uint8_t* mask, const bf16* x0, int n, int D,
                       int H, int W, float* r, float* gout, double* sums, const float* coef) {
    const long long per = (long long)D * H * W;
    const long long vox = (long long)n * per;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double q[4] = {0.0, 0.0, 0.0, 0.0};
    const int smp = (int)(min(v, vox - 1) / per);
    if (v < vox && mask[v]) {
        const int w = (int)(v % W), h = (int)((v / W) % H), d = (int)((v / ((long long)W * H)) % D);
        const long long off[6] = {1, -1, W, -(long long)W, (long long)W * H, -(long long)W * H};
        const bool in[6] = {w + 1 < W, w > 0, h + 1 < H, h > 0, d + 1 < D, d > 0};
        int ns = 0;
        float nb = 0.f;
        const float ev = out[v] - target[v];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (!in[k]) continue;
            const long long u = v + off[k];
            if (!vox_solid(x0, u)) ns++;
            if (mask[u]) nb += GRAD ? r[u] : out[u] - target[u];
        }
        if (GRAD) {
            gout[v] = coef[2 * smp] * ((float)ns * r[v] - nb) + coef[2 * smp + 1] * ev;
        } else {
            const float rv = (float)ns * ev - nb;
            const float bv = __bfloat162float(x0[v * 16]);
            r[v] = rv;
            q[0] = (double)rv * rv;
            q[1] = (double)ev * ev;
            q[2] = (double)target[v] * target[v];
            q[3] = (double)bv * bv;
        }
    } else if (v < vox) {
        if (GRAD) gout[v] = 0.f;
        else r[v] = 0.f;
    }
    if (!GRAD) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            for (int o = 16; o > 0; o >>= 1) q[k] += __shfl_xor_sync(0xffffffffu, q[k], o);
            if ((threadIdx.x & 31) == 0 && q[k] != 0.0) atomicAdd(&sums[4 * smp + k], q[k]);
        }
    }
}

// Loss and gradient factors from the per-sample sums (one warp).  A sample
// whose residual, error, target or rhs is zero contributes nothing to that term.
__global__ void k_loss_coef(const double* sums, int n, float lam, float* coef, double* loss, float* loss_out) {
    double l = 0.0;
    for (int s = threadIdx.x; s < n; s += 32) {
        const double rr = sums[4 * s], ee = sums[4 * s + 1], tt = sums[4 * s + 2], bb = sums[4 * s + 3];
        const double nr = sqrt(rr), nb = sqrt(bb), ne = sqrt(ee), nt = sqrt(tt);
        const bool res_ok = nr > 0.0 && nb > 0.0, err_ok = ne > 0.0 && nt > 0.0;
        coef[2 * s] = res_ok ? (float)(1.0 / (n * nr * nb)) : 0.f;
        coef[2 * s + 1] = err_ok ? (float)(lam / (n * ne * nt)) : 0.f;
        l += (res_ok ? nr / nb : 0.0) + (err_ok ? lam * ne / nt : 0.0);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (threadIdx.x == 0) {
        *loss = l / n;
        if (loss_out) *loss_out = (float)(l / n);
    }
}

// Training batch from a resident pool: sample b of the batch is pool sample
// idx[b].  types: 0 fluid (an unknown of the solve), 1 air, 2 solid; rhs and
// target are the scaled rhs and pressure.  Writes x0 (16 channels: rhs, fluid,
// solid, air, 0...), the batch target and the fluid mask.
__global__ void k_gather_batch(const uint8_t* types, const float* rhs, const float* target, const int* idx,
                               long long per, int batch, bf16* x0, float* tb, uint8_t* mb) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= per * batch) return;
    const long long b = v / per, j = v - b * per;
    const long long src = (long long)idx[b] * per + j;
    const uint8_t t = types[src];
    const float a[8] = {t == 0 ? rhs[src] : 0.f, t == 0 ? 1.f : 0.f, t == 2 ? 1.f : 0.f, t == 1 ? 1.f : 0.f,
                        0.f, 0.f, 0.f, 0.f};
    const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    st8(x0 + v * 16, a);
    st8(x0 + v * 16 + 8, z);
    tb[v] = t == 0 ? target[src] : 0.f;
    mb[v] = t == 0 ? 1 : 0;
}

// head backward: gz = dloss/d(pre-activation of d0), head weight / bias gradients
__global__ void k_head_bwd(const bf16* d0, const float* gout, long long vox, const float* wgt, float scale, bf16* gz,
                           float* gw, float* gb) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ float sw[17][NT_THREADS / 32];
    float contrib[17];
#pragma unroll
    for (int j = 0; j < 17; j++) contrib[j] = 0.f;
    if (v < vox) {
        const float gpre = gout[v] * scale;
        float a[16];
        {
            float x[8], y[8];
            ld8(d0 + v * 16, x);
            ld8(d0 + v * 16 + 8, y);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                a[j] = x[j];
                a[8 + j] = y[j];
            }
        }
        float g0[8], g1[8];
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const float gj = a[j] > 0.f ? gpre * wgt[j] : 0.f;
            if (j < 8) g0[j] = gj;
            else g1[j - 8] = gj;
            contrib[j] = gpre * a[j];
        }
        contrib[16] = gpre;
        st8(gz + v * 16, g0);
        st8(gz + v * 16 + 8, g1);
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 17; j++) {
        float s = contrib[j];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) sw[j][wp] = s;
    }
    __syncthreads();
    if (threadIdx.x < 17) {
        float s = 0.f;
        for (int k = 0; k < NT_THREADS / 32; k++) s += sw[threadIdx.x][k];
        if (threadIdx.x < 16) atomicAdd(gw + threadIdx.x, s);
        else atomicAdd(gb, s);
    }
}

// gb[c] += sum_v g[v][c]   (C in {16, 32, 64})
__global__ void k_bias_grad(const bf16* g, long long vox, int C, float* gb) {
    __shared__ float red[NT_THREADS];
    const int c = threadIdx.x % C, lane = threadIdx.x / C, lanes = NT_THREADS / C;
    float s = 0.f;
    for (long long v = (long long)blockIdx.x * lanes + lane; v < vox; v += (long long)gridDim.x * lanes)
        s += __bfloat162float(g[v * C + c]);
    red[threadIdx.x] = s;
    __syncthreads();
    if (lane == 0) {
        for (int k = 1; k < lanes; k++) s += red[k * C + c];
        atomicAdd(gb + c, s);
    }
}

// ---- optimiser ------------------------------------------------------------
__global__ void k_adam(float* theta, float* grad, float* m, float* v, long long n, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    theta[i] -= lr * mh / (sqrtf(vh) + eps);
    grad[i] = 0.f;
}

// wb[t][n][c] and wt[t][c][n] from the FP32 master [t][n][c]
__global__ void k_pack_weights(const float* w, int taps, int cout, int cin, bf16* wb, bf16* wt) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)taps * cout * cin;
    if (i >= total) return;
    const int c = (int)(i % cin);
    const int nn = (int)((i / cin) % cout);
    const int t = (int)(i / ((long long)cin * cout));
    const bf16 b = __float2bfloat16_rn(w[i]);
    wb[i] = b;
    wt[((long long)t * cin + c) * cout + nn] = b;
}

// ---- solver hook ------------------------------------------------------------
// acc[0] += b^2 over fluid cells, acc[1] += 1
__global__ void k_rhs_stats(GridGeom g, const uint16_t* code, const double* b, double* acc) {
    __shared__ double s0[NT_THREADS / 32], s1[NT_THREADS / 32];
    double a0 = 0.0, a1 = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell;
         c += (long long)gridDim.x * blockDim.x) {
        if (code[c] & CODE_FLUID_BIT) {
            a0 += b[c] * b[c];
            a1 += 1.0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s0[threadIdx.x >> 5] = a0;
        s1[threadIdx.x >> 5] = a1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < NT_THREADS / 32; k++) {
            a0 += s0[k];
            a1 += s1[k];
        }
        atomicAdd(&acc[0], a0);
        atomicAdd(&acc[1], a1);
    }
}

__device__ __forceinline__ double rhs_rms(const double* acc) {
    return acc[1] > 0.0 && acc[0] > 0.0 ? sqrt(acc[0] / acc[1]) : 1.0;
}

// network voxel (d, h, w) = grid cell (x, y, z); volume padded to multiples of 8
__global__ void k_net_input_solver(GridGeom g, const uint16_t* code, const uint8_t* flags, const double* b,
                                   const double* acc, int D, int H, int W, bf16* x0) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= (long long)D * H * W) return;
    const int z = (int)(v % W), y = (int)((v / W) % H), x = (int)(v / ((long long)W * H));
    float a[8] = {0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // outside the grid: solid
    if (x < g.nx && y < g.ny && z < g.nz) {
        const long long c = gidx(g, x, y, z);
        if (code[c] & CODE_FLUID_BIT) {
            a[0] = (float)(b[c] / rhs_rms(acc));
            a[1] = 1.f;
            a[2] = 0.f;
        } else if (flags[c] != C_SOLID) {
            a[2] = 0.f;
            a[3] = 1.f;
        }
    }
    const float zz[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    st8(x0 + v * 16, a);
    st8(x0 + v * 16 + 8, zz);
}

__global__ void k_guess_out(GridGeom g, const uint16_t* code, const float* out, const double* acc, int D, int H,
                            int W, float* guess) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    int x, y, z;
    cell_xyz(g, c, x, y, z);
    float p = 0.f;
    if (z < g.nz && (code[c] & CODE_FLUID_BIT)) p = (float)(out[((long long)x * H + y) * W + z] * rhs_rms(acc));
    guess[c] = p;
}

// ---- host ---------------------------------------------------------------------
struct LayerSpec {
    int taps, cin, cout;
};
constexpr LayerSpec kSpec[NET_LAYERS] = {
    {27, 16, 16}, {27, 16, 16}, {1, 128, 32},  {27, 32, 32}, {27, 32, 32}, {1, 256, 64},
    {27, 64, 64}, {27, 64, 64}, {1, 512, 64},  {27, 64, 64}, {27, 64, 64}, {27, 128, 64},
    {27, 64, 64}, {27, 96, 32}, {27, 32, 32},  {27, 48, 16}, {27, 16, 16}};

// forward tensors
enum {
    X0, A0, CAT0, S2D0, X1, A1, CAT1, S2D1, X2, A2, CAT2, S2D2, X3, A3, B3, C2O, D2, C1O, D1, C0O, D0, NACT
};
constexpr int kActC[NACT] = {16, 16, 48, 128, 32, 32, 96, 256, 64, 64, 128, 512, 64, 64, 64, 64, 64, 32, 32, 16, 16};
constexpr int kActL[NACT] = {0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 2, 2, 1, 1, 0, 0};
// gradient tensors
enum {
    GD0, GC0, GCAT0, GD1, GC1, GCAT1, GD2, GC2, GCAT2, GB3, GA3, GX3, GS2D2, GE2, GA2, GX2, GS2D1, GE1, GA1, GX1,
    GS2D0, GE0, GA0, NGRAD
};
constexpr int kGradC[NGRAD] = {16, 16, 48, 32, 32, 96, 64, 64, 128, 64, 64, 64, 512, 64, 64, 64, 256, 32, 32, 32,
                               128, 16, 16};
constexpr int kGradL[NGRAD] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 3, 2, 2, 2, 2, 1, 1, 1, 1, 0, 0};

// per layer: forward input, output (buffer, channel offset)
constexpr int kIn[NET_LAYERS] = {X0, A0, S2D0, X1, A1, S2D1, X2, A2, S2D2, X3, A3, CAT2, C2O, CAT1, C1O, CAT0, C0O};
constexpr int kOut[NET_LAYERS] = {A0, CAT0, X1, A1, CAT1, X2, A2, CAT2, X3, A3, B3, C2O, D2, C1O, D1, C0O, D0};
constexpr int kOutOff[NET_LAYERS] = {0, 32, 0, 0, 64, 0, 0, 64, 0, 0, 0, 0, 0, 0, 0, 0, 0};
// per layer: gradient of its pre-activation, gradient of its input (or -1), input mask (or -1)
constexpr int kGz[NET_LAYERS] = {GA0, GE0, GX1, GA1, GE1, GX2, GA2, GE2, GX3, GA3, GB3, GC2, GD2, GC1, GD1, GC0, GD0};
constexpr int kGin[NET_LAYERS] = {-1, GA0, GS2D0, GX1, GA1, GS2D1, GX2, GA2, GS2D2, GX3, GA3, GCAT2, GC2, GCAT1, GC1,
                                  GCAT0, GC0};
constexpr int kGinMask[NET_LAYERS] = {-1, A0, -1, X1, A1, -1, X2, A2, -1, X3, A3, -1, C2O, -1, C1O, -1, C0O};

long long level_vox(const NetShape& s, int l) {
    return (long long)s.n * (s.d >> l) * (s.h >> l) * (s.w >> l);
}

int fail(fsim_net* net, const std::string& msg, int code) {
    net->err = msg;
    return code;
}

#define NET_TRY(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return fail(net, std::string(#call) + ": " + cudaGetErrorString(e_), FSIM_E_CUDA); \
    } while (0)

unsigned nblk(long long n) { return (unsigned)((n + NT_THREADS - 1) / NT_THREADS); }

int pack_all_weights(fsim_net* net) {
    for (int l = 0; l < NET_LAYERS; l++) {
        const NetLayer& L = net->L[l];
        const long long tot = (long long)L.taps * L.cout * L.cin;
        k_pack_weights<<<nblk(tot), NT_THREADS, 0, net->stream>>>(net->theta + L.w_off, L.taps, L.cout, L.cin, L.wb,
                                                                  L.wt);
    }
    net->launches += NET_LAYERS;
    NET_TRY(cudaGetLastError());
    return FSIM_OK;
}

void free_ws(fsim_net* net) {
    if (net->ws) cudaFree(net->ws);
    net->ws = nullptr;
    net->ws_bytes = 0;
    net->act.clear();
    net->gbuf.clear();
    net->amap.clear();
    net->out = nullptr;
    net->res = nullptr;
    net->gout = nullptr;
    net->shape = NetShape{};
}

int ensure_ws(fsim_net* net, int n, int d, int h, int w, bool train) {
    if (n <= 0 || d <= 0 || h <= 0 || w <= 0 || d % 8 || h % 8 || w % 8)
        return fail(net, "network volume must be positive multiples of 8", FSIM_E_INVALID);
    NetShape s{n, d, h, w, train};
    if (net->ws && net->shape.n == n && net->shape.d == d && net->shape.h == h && net->shape.w == w &&
        (net->shape.train || !train))
        return FSIM_OK;
    free_ws(net);
    size_t bytes = 0;
    auto take = [&](size_t b) {
        const size_t off = bytes;
        bytes += (b + 255) & ~(size_t)255;
        return off;
    };
    std::vector<size_t> aoff(NACT), goff(NGRAD);
    for (int i = 0; i < NACT; i++) aoff[i] = take((size_t)level_vox(s, kActL[i]) * kActC[i] * 2);
    if (train)
        for (int i = 0; i < NGRAD; i++) goff[i] = take((size_t)level_vox(s, kGradL[i]) * kGradC[i] * 2);
    size_t res_off = 0, gout_off = 0, tb_off = 0, mb_off = 0;
    if (train) {
        res_off = take((size_t)level_vox(s, 0) * 4);
        gout_off = take((size_t)level_vox(s, 0) * 4);
        tb_off = take((size_t)level_vox(s, 0) * 4);
        mb_off = take((size_t)level_vox(s, 0));
    }
    const size_t out_off = take((size_t)level_vox(s, 0) * 4);
    void* mem = nullptr;
    NET_TRY(cudaMalloc(&mem, bytes));
    net->ws = mem;
    net->ws_bytes = bytes;
    net->shape = s;
    char* base = (char*)mem;
    net->act.resize(NACT);
    for (int i = 0; i < NACT; i++) net->act[i] = NetBuf{(bf16*)(base + aoff[i]), kActC[i], kActL[i]};
    if (train) {
        net->gbuf.resize(NGRAD);
        for (int i = 0; i < NGRAD; i++) net->gbuf[i] = NetBuf{(bf16*)(base + goff[i]), kGradC[i], kGradL[i]};
        // slices of the concatenation gradients that no kernel writes stay defined
        NET_TRY(cudaMemsetAsync(base + goff[0], 0, out_off - goff[0], net->stream));
    }
    net->out = (float*)(base + out_off);
    net->res = train ? (float*)(base + res_off) : nullptr;
    net->gout = train ? (float*)(base + gout_off) : nullptr;
    net->batch_target = train ? (float*)(base + tb_off) : nullptr;
    net->batch_mask = train ? (uint8_t*)(base + mb_off) : nullptr;
    net->amap.resize(2 * NET_LAYERS);
    for (int l = 0; l < NET_LAYERS; l++) {
        const NetBuf& in = net->act[kIn[l]];
        const int lv = in.lev;
        if (!conv_act_map(&net->amap[l], in.p, n, d >> lv, h >> lv, w >> lv, in.c, net->L[l].taps))
            return fail(net, "tensor map of a network activation failed", FSIM_E_CUDA);
        if (train && l > 0) {
            const NetBuf& gz = net->gbuf[kGz[l]];
            if (!conv_act_map(&net->amap[NET_LAYERS + l], gz.p, n, d >> gz.lev, h >> gz.lev, w >> gz.lev, gz.c,
                              net->L[l].taps))
                return fail(net, "tensor map of a network gradient failed", FSIM_E_CUDA);
        }
    }
    return FSIM_OK;
}

int conv_fwd(fsim_net* net, int l) {
    const NetLayer& L = net->L[l];
    const NetBuf& out = net->act[kOut[l]];
    const int lv = out.lev;
    ConvLaunch c{};
    c.taps = L.taps;
    c.n = net->shape.n;
    c.d = net->shape.d >> lv;
    c.h = net->shape.h >> lv;
    c.w = net->shape.w >> lv;
    c.cin = L.cin;
    c.cout = L.cout;
    c.flip = 0;
    c.bias = net->theta + L.b_off;
    c.relu = 1;
    c.y = out.p;
    c.ys = out.c;
    c.yo = kOutOff[l];
    c.err = net->d_err;
    c.mx = &net->amap[l];
    c.mw = &L.mw;
    net->launches++;
    return launch_conv_mma(c, net->stream);
}

int s2d(fsim_net* net, int src, int so, int C, int dst) {
    const NetBuf& s = net->act[src];
    const int lv = s.lev;
    const NetShape& sh = net->shape;
    const long long total = level_vox(sh, lv + 1) * 8 * (C / 8);
    k_s2d<<<nblk(total), NT_THREADS, 0, net->stream>>>(s.p, s.c, so, C, sh.n, sh.d >> lv, sh.h >> lv, sh.w >> lv,
                                                       net->act[dst].p);
    net->launches++;
    return FSIM_OK;
}

int upsample(fsim_net* net, int src, int dst) {
    const NetBuf& s = net->act[src];
    const int lv = s.lev;
    const NetShape& sh = net->shape;
    const long long total = level_vox(sh, lv) * (s.c / 8);
    if (total >= (1ll << 31)) return fail(net, "up-sampling volume too large", FSIM_E_CAPACITY);
    k_upsample<<<nblk(total), NT_THREADS, 0, net->stream>>>(s.p, s.c, sh.n, sh.d >> lv, sh.h >> lv, sh.w >> lv,
                                                            net->act[dst].p, net->act[dst].c);
    net->launches++;
    return FSIM_OK;
}

}  // namespace

int net_forward(fsim_net* net) {
    int rc;
    auto conv = [&](int l) { return (rc = conv_fwd(net, l)) == FSIM_OK; };
    if (!conv(0) || !conv(1)) return rc;
    s2d(net, CAT0, 32, 16, S2D0);
    if (!conv(2) || !conv(3) || !conv(4)) return rc;
    s2d(net, CAT1, 64, 32, S2D1);
    if (!conv(5) || !conv(6) || !conv(7)) return rc;
    s2d(net, CAT2, 64, 64, S2D2);
    if (!conv(8) || !conv(9) || !conv(10)) return rc;
    upsample(net, B3, CAT2);
    if (!conv(11) || !conv(12)) return rc;
    upsample(net, D2, CAT1);
    if (!conv(13) || !conv(14)) return rc;
    upsample(net, D1, CAT0);
    if (!conv(15) || !conv(16)) return rc;
    const long long vox = level_vox(net->shape, 0);
    k_head<<<nblk(vox), NT_THREADS, 0, net->stream>>>(net->act[D0].p, vox, net->theta + net->head_w,
                                                      net->theta + net->head_b, net->out_scale, net->out);
    net->launches++;
    NET_TRY(cudaGetLastError());
    return FSIM_OK;
}

namespace {

int conv_bwd(fsim_net* net, int l) {
    const NetLayer& L = net->L[l];
    const NetBuf& gz = net->gbuf[kGz[l]];
    const NetBuf& x = net->act[kIn[l]];
    const NetShape& sh = net->shape;
    const int lv = gz.lev;
    // weight gradient
    WgradLaunch wg{};
    wg.taps = L.taps;
    wg.n = sh.n;
    wg.d = sh.d >> lv;
    wg.h = sh.h >> lv;
    wg.w = sh.w >> lv;
    wg.cin = L.cin;
    wg.cout = L.cout;
    wg.x = x.p;
    wg.g = gz.p;
    wg.dw = net->grad + L.w_off;
    wg.err = net->d_err;
    int rc = launch_conv_wgrad(wg, net->stream);
    if (rc) return fail(net, "weight-gradient launch failed", rc);
    const long long vox = level_vox(sh, lv);
    int bl = (int)std::min<long long>((vox + 255) / 256, 1024);
    k_bias_grad<<<bl, NT_THREADS, 0, net->stream>>>(gz.p, vox, L.cout, net->grad + L.b_off);
    net->launches += 2;
    if (kGin[l] < 0) return FSIM_OK;
    // input gradient
    const NetBuf& gi = net->gbuf[kGin[l]];
    ConvLaunch c{};
    c.taps = L.taps;
    c.n = sh.n;
    c.d = sh.d >> lv;
    c.h = sh.h >> lv;
    c.w = sh.w >> lv;
    c.cin = L.cout;
    c.cout = L.cin;
    c.flip = L.taps == 27 ? 1 : 0;
    c.bias = nullptr;
    c.relu = 0;
    if (kGinMask[l] >= 0) {
        c.mask = net->act[kGinMask[l]].p;
        c.ms = net->act[kGinMask[l]].c;
        c.mo = 0;
    }
    c.y = gi.p;
    c.ys = gi.c;
    c.yo = 0;
    c.err = net->d_err;
    c.mx = &net->amap[NET_LAYERS + l];
    c.mw = &L.mwt;
    net->launches++;
    rc = launch_conv_mma(c, net->stream);
    if (rc) return fail(net, "input-gradient launch failed", rc);
    return FSIM_OK;
}

int up_bwd(fsim_net* net, int gcat, int mask, int out) {
    const NetBuf& m = net->act[mask];
    const int lv = m.lev;
    const NetShape& sh = net->shape;
    const long long total = level_vox(sh, lv) * (m.c / 8);
    k_upsample_bwd<<<nblk(total), NT_THREADS, 0, net->stream>>>(net->gbuf[gcat].p, net->gbuf[gcat].c, m.p, m.c, sh.n,
                                                                sh.d >> lv, sh.h >> lv, sh.w >> lv,
                                                                net->gbuf[out].p);
    net->launches++;
    return FSIM_OK;
}

int d2s(fsim_net* net, int gs2d, int gcat, int cat, int off, int C, int out) {
    const NetBuf& gc = net->gbuf[gcat];
    const int lv = gc.lev;
    const NetShape& sh = net->shape;
    const long long total = level_vox(sh, lv) * (C / 8);
    k_d2s_add_mask<<<nblk(total), NT_THREADS, 0, net->stream>>>(net->gbuf[gs2d].p, gc.p, gc.c, off, net->act[cat].p,
                                                                net->act[cat].c, off, C, sh.n, sh.d >> lv,
                                                                sh.h >> lv, sh.w >> lv, net->gbuf[out].p);
    net->launches++;
    return FSIM_OK;
}

int net_backward(fsim_net* net, const float* target, const uint8_t* mask, float* loss_out = nullptr) {
    const long long vox = level_vox(net->shape, 0);
    const NetShape& sh = net->shape;
    if (sh.n > NET_MAX_BATCH) return fail(net, "training batch larger than 64 samples", FSIM_E_INVALID);
    NET_TRY(cudaMemsetAsync(net->d_sums, 0, sizeof(double) * 4 * sh.n, net->stream));
    k_loss<false><<<nblk(vox), NT_THREADS, 0, net->stream>>>(net->out, target, mask, net->act[X0].p, sh.n, sh.d, sh.h,
                                                             sh.w, net->res, nullptr, net->d_sums, nullptr);
    k_loss_coef<<<1, 32, 0, net->stream>>>(net->d_sums, sh.n, net->loss_l2_weight, net->d_coef, net->d_loss,
                                           loss_out);
    k_loss<true><<<nblk(vox), NT_THREADS, 0, net->stream>>>(net->out, target, mask, net->act[X0].p, sh.n, sh.d, sh.h,
                                                            sh.w, net->res, net->gout, nullptr, net->d_coef);
    k_head_bwd<<<nblk(vox), NT_THREADS, 0, net->stream>>>(net->act[D0].p, net->gout, vox, net->theta + net->head_w,
                                                          net->out_scale, net->gbuf[GD0].p, net->grad + net->head_w,
                                                          net->grad + net->head_b);
    net->launches += 4;
    int rc;
    auto cb = [&](int l) { return (rc = conv_bwd(net, l)) == FSIM_OK; };
    if (!cb(16) || !cb(15)) return rc;
    up_bwd(net, GCAT0, D1, GD1);
    if (!cb(14) || !cb(13)) return rc;
    up_bwd(net, GCAT1, D2, GD2);
    if (!cb(12) || !cb(11)) return rc;
    up_bwd(net, GCAT2, B3, GB3);
    if (!cb(10) || !cb(9) || !cb(8)) return rc;
    d2s(net, GS2D2, GCAT2, CAT2, 64, 64, GE2);
    if (!cb(7) || !cb(6) || !cb(5)) return rc;
    d2s(net, GS2D1, GCAT1, CAT1, 64, 32, GE1);
    if (!cb(4) || !cb(3) || !cb(2)) return rc;
    d2s(net, GS2D0, GCAT0, CAT0, 32, 16, GE0);
    if (!cb(1) || !cb(0)) return rc;
    NET_TRY(cudaGetLastError());
    return FSIM_OK;
}

int check_err(fsim_net* net) {
    unsigned e = 0;
    NET_TRY(cudaMemcpyAsync(&e, net->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, net->stream));
    NET_TRY(cudaStreamSynchronize(net->stream));
    if (e) {
        NET_TRY(cudaMemsetAsync(net->d_err, 0, sizeof(unsigned), net->stream));
        return fail(net, "a tensor-core convolution gave up waiting for its operands (error bits " +
                             std::to_string(e) + ")",
                    FSIM_E_TIMEOUT);
    }
    return FSIM_OK;
}

// host copy / device pointer helper: returns a device pointer to n bytes of src
struct Staged {
    void* p = nullptr;
    bool owned = false;
};
int stage_in(fsim_net* net, const void* src, size_t bytes, int where, Staged& out) {
    if (where == FSIM_DEVICE) {
        out.p = const_cast<void*>(src);
        out.owned = false;
        return FSIM_OK;
    }
    NET_TRY(cudaMallocAsync(&out.p, bytes, net->stream));
    out.owned = true;
    NET_TRY(cudaMemcpyAsync(out.p, src, bytes, cudaMemcpyHostToDevice, net->stream));
    return FSIM_OK;
}
void unstage(fsim_net* net, Staged& s) {
    if (s.owned && s.p) cudaFreeAsync(s.p, net->stream);
    s = Staged{};
}

// Gaussian from two SplitMix64 uniforms (Box-Muller)
double gauss(uint64_t seed, uint64_t i) {
    const double u1 = uniform01(seed, 2 * i) * (1.0 - 1e-12) + 1e-12;
    const double u2 = uniform01(seed, 2 * i + 1);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

}  // namespace

int net_guess(fsim_net* net, const GridGeom& g, const uint16_t* code, const uint8_t* flags, const double* b,
              float* guess, cudaStream_t s) {
    const int D = (g.nx + 7) / 8 * 8, H = (g.ny + 7) / 8 * 8, W = (g.nz + 7) / 8 * 8;
    cudaStream_t keep = net->stream;
    net->stream = s;
    int rc = ensure_ws(net, 1, D, H, W, net->shape.train);
    if (rc) {
        net->stream = keep;
        return rc;
    }
    cudaMemsetAsync(net->d_rms, 0, 2 * sizeof(double), s);
    k_rhs_stats<<<4 * 152, NT_THREADS, 0, s>>>(g, code, b, net->d_rms);
    const long long vox = (long long)D * H * W;
    k_net_input_solver<<<nblk(vox), NT_THREADS, 0, s>>>(g, code, flags, b, net->d_rms, D, H, W, net->act[X0].p);
    net->launches += 2;
    rc = net_forward(net);
    if (rc == FSIM_OK) {
        k_guess_out<<<nblk(g.ncell), NT_THREADS, 0, s>>>(g, code, net->out, net->d_rms, D, H, W, guess);
        net->launches++;
        if (cudaGetLastError() != cudaSuccess) rc = fail(net, "guess output launch failed", FSIM_E_CUDA);
    }
    net->stream = keep;
    return rc;
}

extern "C" {

int fsim_net_create(uint64_t seed, float out_scale, fsim_net** out) {
    if (!out) return FSIM_E_INVALID;
    *out = nullptr;
    fsim_net* net = new fsim_net();
    net->out_scale = out_scale > 0.f ? out_scale : 1.f;
    long long off = 0;
    for (int l = 0; l < NET_LAYERS; l++) {
        NetLayer& L = net->L[l];
        L.taps = kSpec[l].taps;
        L.cin = kSpec[l].cin;
        L.cout = kSpec[l].cout;
        L.w_off = off;
        off += (long long)L.taps * L.cin * L.cout;
        L.b_off = off;
        off += L.cout;
    }
    net->head_w = off;
    off += 16;
    net->head_b = off;
    off += 1;
    net->nparams = off;
    auto bad = [&](const char* what) {
        net->err = what;
        fsim_net_destroy(net);
        return FSIM_E_CUDA;
    };
    if (cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) != cudaSuccess) return bad("stream");
    const size_t pb = (size_t)off * 4;
    if (cudaMalloc(&net->theta, pb) != cudaSuccess || cudaMalloc(&net->grad, pb) != cudaSuccess ||
        cudaMalloc(&net->adam_m, pb) != cudaSuccess || cudaMalloc(&net->adam_v, pb) != cudaSuccess ||
        cudaMalloc(&net->d_err, 64) != cudaSuccess || cudaMalloc(&net->d_loss, 8) != cudaSuccess ||
        cudaMalloc(&net->d_sums, sizeof(double) * 4 * NET_MAX_BATCH) != cudaSuccess ||
        cudaMalloc(&net->d_coef, sizeof(float) * 2 * NET_MAX_BATCH) != cudaSuccess ||
        cudaMalloc(&net->d_rms, 16) != cudaSuccess)
        return bad("parameter allocation");
    long long wtot = 0;
    for (int l = 0; l < NET_LAYERS; l++) wtot += ((long long)net->L[l].taps * net->L[l].cin * net->L[l].cout + 127) / 128 * 128;
    if (cudaMalloc(&net->wpool, (size_t)wtot * 2 * 2) != cudaSuccess) return bad("weight allocation");
    bf16* wp = net->wpool;
    for (int l = 0; l < NET_LAYERS; l++) {
        NetLayer& L = net->L[l];
        const long long cnt = ((long long)L.taps * L.cin * L.cout + 127) / 128 * 128;
        L.wb = wp;
        wp += cnt;
        L.wt = wp;
        wp += cnt;
        if (!conv_wt_map(&L.mw, L.wb, L.taps, L.cout, L.cin, conv_nt(L.taps, L.cout)) ||
            !conv_wt_map(&L.mwt, L.wt, L.taps, L.cin, L.cout, conv_nt(L.taps, L.cin)))
            return bad("weight tensor maps");
    }
    // He initialisation (fan-in of the real inputs), zero biases, zero head
    std::vector<float> h((size_t)off, 0.f);
    uint64_t k = 0;
    for (int l = 0; l < NET_LAYERS; l++) {
        const NetLayer& L = net->L[l];
        const int cin_real = l == 0 ? 4 : L.cin;
        const double sd = std::sqrt(2.0 / ((double)L.taps * cin_real));
        for (long long i = 0; i < (long long)L.taps * L.cin * L.cout; i++) {
            const int c = (int)(i % L.cin);
            h[(size_t)(L.w_off + i)] = (l == 0 && c >= 4) ? 0.f : (float)(sd * gauss(seed, k++));
        }
    }
    // the head starts at zero: the untrained network predicts the zero guess,
    // so training (residual loss) starts from the zero start's loss and improves on it
    for (int c = 0; c < 16; c++) h[(size_t)(net->head_w + c)] = 0.f;
    if (cudaMemcpy(net->theta, h.data(), pb, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(net->grad, 0, pb) != cudaSuccess || cudaMemset(net->adam_m, 0, pb) != cudaSuccess ||
        cudaMemset(net->adam_v, 0, pb) != cudaSuccess || cudaMemset(net->d_err, 0, 64) != cudaSuccess)
        return bad("parameter upload");
    if (pack_all_weights(net) != FSIM_OK || cudaStreamSynchronize(net->stream) != cudaSuccess)
        return bad("weight packing");
    *out = net;
    return FSIM_OK;
}

int fsim_net_destroy(fsim_net* net) {
    if (!net) return FSIM_OK;
    if (net->stream) cudaStreamSynchronize(net->stream);
    free_ws(net);
    cudaFree(net->theta);
    cudaFree(net->grad);
    cudaFree(net->adam_m);
    cudaFree(net->adam_v);
    cudaFree(net->d_err);
    cudaFree(net->d_loss);
    cudaFree(net->d_sums);
    cudaFree(net->d_coef);
    cudaFree(net->d_rms);
    cudaFree(net->wpool);
    if (net->stream) cudaStreamDestroy(net->stream);
    delete net;
    return FSIM_OK;
}

namespace {
thread_local std::string g_conv_err;  // last fsim_net_conv failure on this thread
}
const char* fsim_net_last_error(const fsim_net* net) { return net ? net->err.c_str() : g_conv_err.c_str(); }

int64_t fsim_net_num_params(const fsim_net* net) { return net ? net->nparams : 0; }

int fsim_net_get_params(fsim_net* net, float* dst, int what, int where) {
    if (!net || !dst || what < 0 || what > 1) return FSIM_E_INVALID;
    const float* src = what == 0 ? net->theta : net->grad;
    NET_TRY(cudaMemcpyAsync(dst, src, (size_t)net->nparams * 4,
                            where == FSIM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, net->stream));
    NET_TRY(cudaStreamSynchronize(net->stream));
    return FSIM_OK;
}

int fsim_net_set_params(fsim_net* net, const float* src, int where) {
    if (!net || !src) return FSIM_E_INVALID;
    NET_TRY(cudaMemcpyAsync(net->theta, src, (size_t)net->nparams * 4,
                            where == FSIM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, net->stream));
    int rc = pack_all_weights(net);
    if (rc) return rc;
    NET_TRY(cudaStreamSynchronize(net->stream));
    return FSIM_OK;
}

int fsim_net_forward(fsim_net* net, int n, int d, int h, int w, const float* in, float* out, int train, int where) {
    if (!net || !in) return FSIM_E_INVALID;
    int rc = ensure_ws(net, n, d, h, w, train != 0);
    if (rc) return rc;
    const long long vox = (long long)n * d * h * w;
    Staged sin;
    if ((rc = stage_in(net, in, (size_t)vox * 16, where, sin))) return rc;
    k_pack_input<<<nblk(vox), NT_THREADS, 0, net->stream>>>((const float*)sin.p, vox, net->act[X0].p);
    net->launches++;
    rc = net_forward(net);
    unstage(net, sin);
    if (rc) return rc;
    if (out) {
        NET_TRY(cudaMemcpyAsync(out, net->out, (size_t)vox * 4,
                                where == FSIM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                net->stream));
    }
    return check_err(net);
}

int fsim_net_backward(fsim_net* net, const float* target, const uint8_t* mask, float* loss, int where) {
    if (!net || !target || !mask) return FSIM_E_INVALID;
    if (!net->ws || !net->shape.train) return fail(net, "fsim_net_backward needs a training forward pass", FSIM_E_STATE);
    const long long vox = level_vox(net->shape, 0);
    Staged st, sm;
    int rc;
    if ((rc = stage_in(net, target, (size_t)vox * 4, where, st))) return rc;
    if ((rc = stage_in(net, mask, (size_t)vox, where, sm))) {
        unstage(net, st);
        return rc;
    }
    rc = net_backward(net, (const float*)st.p, (const uint8_t*)sm.p);
    unstage(net, st);
    unstage(net, sm);
    if (rc) return rc;
    if ((rc = check_err(net))) return rc;
    if (loss) {
        double l = 0.0;
        NET_TRY(cudaMemcpy(&l, net->d_loss, sizeof(double), cudaMemcpyDeviceToHost));
        *loss = (float)l;
    }
    return FSIM_OK;
}

int fsim_net_set_loss(fsim_net* net, float l2_weight) {
    if (!net || !(l2_weight >= 0.f)) return FSIM_E_INVALID;
    net->loss_l2_weight = l2_weight;
    return FSIM_OK;
}

int fsim_net_train_batch(fsim_net* net, int d, int h, int w, const uint8_t* types, const float* rhs,
                         const float* target, const int* idx, int batch, float lr, float* loss_out) {
    if (!net || !types || !rhs || !target || !idx || batch <= 0 || batch > NET_MAX_BATCH || !(lr > 0.f))
        return FSIM_E_INVALID;
    int rc = ensure_ws(net, batch, d, h, w, true);
    if (rc) return rc;
    const long long per = (long long)d * h * w;
    k_gather_batch<<<nblk(per * batch), NT_THREADS, 0, net->stream>>>(types, rhs, target, idx, per, batch,
                                                                      net->act[X0].p, net->batch_target,
                                                                      net->batch_mask);
    net->launches++;
    NET_TRY(cudaGetLastError());
    if ((rc = net_forward(net))) return rc;
    NET_TRY(cudaMemsetAsync(net->grad, 0, (size_t)net->nparams * 4, net->stream));
    if ((rc = net_backward(net, net->batch_target, net->batch_mask, loss_out))) return rc;
    return fsim_net_adam(net, lr);
}

int fsim_net_zero_grad(fsim_net* net) {
    if (!net) return FSIM_E_INVALID;
    NET_TRY(cudaMemsetAsync(net->grad, 0, (size_t)net->nparams * 4, net->stream));
    return FSIM_OK;
}

int fsim_net_adam(fsim_net* net, float lr) {
    if (!net || !(lr > 0.f)) return FSIM_E_INVALID;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    net->adam_t++;
    const float bc1 = (float)(1.0 - std::pow((double)b1, (double)net->adam_t));
    const float bc2 = (float)(1.0 - std::pow((double)b2, (double)net->adam_t));
    k_adam<<<nblk(net->nparams), NT_THREADS, 0, net->stream>>>(net->theta, net->grad, net->adam_m, net->adam_v,
                                                               net->nparams, lr, b1, b2, eps, bc1, bc2);
    net->launches++;
    int rc = pack_all_weights(net);
    if (rc) return rc;
    NET_TRY(cudaGetLastError());
    return FSIM_OK;
}

int fsim_net_train_step(fsim_net* net, int n, int d, int h, int w, const float* in, const float* target,
                        const uint8_t* mask, float lr, float* loss, int where) {
    int rc = fsim_net_forward(net, n, d, h, w, in, nullptr, 1, where);
    if (rc) return rc;
    if ((rc = fsim_net_backward(net, target, mask, loss, where))) return rc;
    return fsim_net_adam(net, lr);
}

int fsim_net_synchronize(fsim_net* net) {
    if (!net) return FSIM_E_INVALID;
    NET_TRY(cudaStreamSynchronize(net->stream));
    return check_err(net);
}

int fsim_net_conv(int taps, int mode, int n, int d, int h, int w, int cin, int cout, const float* x,
                  const float* wgt, const float* g, float* out, int where) {
    if ((taps != 27 && taps != 1) || mode < 0 || mode > 2 || n <= 0 || d <= 0 || h <= 0 || w <= 0 || cin % 16 ||
        cout % 16 || cin <= 0 || cout <= 0)
        return FSIM_E_INVALID;
    if ((mode != 1 && !x) || (mode != 2 && !wgt) || (mode != 0 && !g) || !out) return FSIM_E_INVALID;
    const long long vox = (long long)n * d * h * w;
    const long long nw = (long long)taps * cin * cout;
    if (mode == 2 && cout > 64) return FSIM_E_INVALID;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return FSIM_E_CUDA;
    const cudaMemcpyKind h2d = where == FSIM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind d2h = where == FSIM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    float *fx = nullptr, *fw = nullptr, *fg = nullptr, *fo = nullptr;
    bf16 *bx = nullptr, *bw = nullptr, *bwt = nullptr, *bg = nullptr, *bo = nullptr;
    unsigned* err = nullptr;
    const long long nout = mode == 0 ? vox * cout : mode == 1 ? vox * cin : nw;
    int rc = FSIM_OK;
    g_conv_err.clear();
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == FSIM_OK) {
            rc = FSIM_E_CUDA;
            g_conv_err = cudaGetErrorString(e);
        }
        return rc == FSIM_OK;
    };
    ok(cudaMalloc(&err, 16));
    ok(cudaMemsetAsync(err, 0, 16, s));
    ok(cudaMalloc(&fo, (size_t)nout * 4));
    if (x) {
        ok(cudaMalloc(&fx, (size_t)vox * cin * 4));
        ok(cudaMalloc(&bx, (size_t)vox * cin * 2));
        ok(cudaMemcpyAsync(fx, x, (size_t)vox * cin * 4, h2d, s));
    }
    if (g) {
        ok(cudaMalloc(&fg, (size_t)vox * cout * 4));
        ok(cudaMalloc(&bg, (size_t)vox * cout * 2));
        ok(cudaMemcpyAsync(fg, g, (size_t)vox * cout * 4, h2d, s));
    }
    if (wgt) {
        ok(cudaMalloc(&fw, (size_t)nw * 4));
        ok(cudaMalloc(&bw, (size_t)nw * 2));
        ok(cudaMalloc(&bwt, (size_t)nw * 2));
        ok(cudaMemcpyAsync(fw, wgt, (size_t)nw * 4, h2d, s));
    }
    if (mode != 2) ok(cudaMalloc(&bo, (size_t)nout * 2));
    if (rc == FSIM_OK) {
        if (x) k_to_bf16<<<nblk(vox * cin), NT_THREADS, 0, s>>>(fx, vox * cin, bx);
        if (g) k_to_bf16<<<nblk(vox * cout), NT_THREADS, 0, s>>>(fg, vox * cout, bg);
        if (wgt) k_pack_weights<<<nblk(nw), NT_THREADS, 0, s>>>(fw, taps, cout, cin, bw, bwt);
        CUtensorMap mx, mw;
        if (mode == 0 || mode == 1) {
            const bool m0 = mode == 0;
            const int kin = m0 ? cin : cout, kout = m0 ? cout : cin;
            if (!conv_act_map(&mx, m0 ? bx : bg, n, d, h, w, kin, taps) ||
                !conv_wt_map(&mw, m0 ? bw : bwt, taps, kout, kin, conv_nt(taps, kout))) {
                rc = FSIM_E_CUDA;
                g_conv_err = "tensor map encoding failed";
            } else {
                ConvLaunch c{};
                c.taps = taps;
                c.n = n; c.d = d; c.h = h; c.w = w;
                c.cin = kin;
                c.cout = kout;
                c.flip = (!m0 && taps == 27) ? 1 : 0;
                c.y = bo;
                c.ys = kout;
                c.yo = 0;
                c.err = err;
                c.mx = &mx;
                c.mw = &mw;
                rc = launch_conv_mma(c, s);
                if (rc) g_conv_err = std::string("convolution launch: ") + cudaGetErrorString(cudaGetLastError());
                if (rc == FSIM_OK) k_to_f32<<<nblk(nout), NT_THREADS, 0, s>>>(bo, nout, fo);
            }
        } else {
            ok(cudaMemsetAsync(fo, 0, (size_t)nout * 4, s));
            WgradLaunch L{};
            L.taps = taps;
            L.n = n; L.d = d; L.h = h; L.w = w;
            L.cin = cin;
            L.cout = cout;
            L.x = bx;
            L.g = bg;
            L.dw = fo;
            L.err = err;
            if (rc == FSIM_OK) rc = launch_conv_wgrad(L, s);
            if (rc) g_conv_err = std::string("weight-gradient launch: ") + cudaGetErrorString(cudaGetLastError());
        }
    }
    if (rc == FSIM_OK) ok(cudaMemcpyAsync(out, fo, (size_t)nout * 4, d2h, s));
    unsigned e = 0;
    if (err) cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s);
    const cudaError_t se = cudaStreamSynchronize(s);
    if (se != cudaSuccess && rc == FSIM_OK) {
        rc = FSIM_E_CUDA;
        g_conv_err = cudaGetErrorString(se);
    }
    if (rc == FSIM_OK && e) {
        rc = FSIM_E_TIMEOUT;
        g_conv_err = "a bounded wait in the convolution gave up";
    }
    cudaFree(fx); cudaFree(fw); cudaFree(fg); cudaFree(fo);
    cudaFree(bx); cudaFree(bw); cudaFree(bwt); cudaFree(bg); cudaFree(bo); cudaFree(err);
    cudaStreamDestroy(s);
    return rc;
}

}  // extern "C"
