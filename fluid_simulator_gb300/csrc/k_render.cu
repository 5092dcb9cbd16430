// k_render.cu -- headless screen-space fluid renderer (include/fsim_render.h).
//
// The passes of FluidSurfaceGfx::render (fluidSurfaceGfx.cpp:81-204) as CUDA
// kernels over device images (row 0 at the bottom, as OpenGL's window):
//   1. sprite depth splat of the surface particles (particle_sprites.vs +
//      particle_sprites_depth.fs): one thread per particle walks the pixels of
//      its billboard, finds the sprite coordinate of each pixel centre by
//      intersecting the pixel's eye ray with the billboard plane (what
//      perspective-correct interpolation of texCoord gives), and keeps the
//      nearest sphere depth with an atomicMin on the depth bits;
//   2. separable Gaussian (gaussian.fs) or bilateral (bilateral.fs) smoothing,
//      x then y, one thread per pixel;
//   3. spray particles (density below the threshold) splatted onto the
//      smoothed depth;
//   4. additive thickness splat (particle_sprites_thickness.fs) depth-tested
//      against the scene -- computed by passes 1 and 3 from the same fragments,
//      which cover every particle once -- then its separable blur
//      (gaussian_thickness.fs);
//   5. normals from the smoothed depth (normal_depth.fs);
//   6. Blinn-Phong shading with Perlin surface noise and thickness
//      transparency, blended over the background (shadedDepth.fs).
// All arithmetic is FP32 like the shaders; this file is compiled without FMA
// contraction so that the C restatement in oracle/ rounds the same way.
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/fsim_render.h"
#include "fsim_common.cuh"

struct fsim_renderer {
    int W = 0, H = 0;
    cudaStream_t own = nullptr;
    float* raw = nullptr;     // sprite depth (before smoothing)
    float* depth = nullptr;   // smoothed depth + spray
    float* tmp = nullptr;     // blur scratch
    float* thick = nullptr;   // thickness
    float* ttmp = nullptr;    // thickness blur scratch
    float4* nd = nullptr;     // normal + depth
    float4* color = nullptr;  // composited frame
    fsim_particle_gfx* parts = nullptr;  // staging for host particles / fsim_render_ctx
    long long parts_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t last = nullptr;
    int launches = 0;
    bool timed = false;
    std::string err;
};

namespace {

struct Mat4 {
    float m[16];  // column-major: m[c * 4 + r]
};

struct Cam {
    Mat4 view, view_inv, proj, proj_inv;
    float pos[4];
};

__device__ __forceinline__ void mul4(const Mat4& M, const float (&v)[4], float (&o)[4]) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
        float s = M.m[r] * v[0];
        s = s + M.m[4 + r] * v[1];
        s = s + M.m[8 + r] * v[2];
        s = s + M.m[12 + r] * v[3];
        o[r] = s;
    }
}

__device__ __forceinline__ float dot3(const float* a, const float* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__device__ __forceinline__ void cross3(const float* a, const float* b, float* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// GLSL normalize; a zero vector stays zero (GLSL leaves it undefined)
__device__ __forceinline__ void normalize3(float* v) {
    const float l = sqrtf(dot3(v, v));
    if (l > 0.f) {
        v[0] = v[0] / l;
        v[1] = v[1] / l;
        v[2] = v[2] / l;
    }
}

// uvToEye: window (texCoord, depth) -> eye-space position
__device__ __forceinline__ void uv_to_eye(const Cam& c, float u, float v, float d, float* e) {
    const float ndc[4] = {u * 2.f - 1.f, v * 2.f - 1.f, d * 2.f - 1.f, 1.f};
    float o[4];
    mul4(c.proj_inv, ndc, o);
    e[0] = o[0] / o[3];
    e[1] = o[1] / o[3];
    e[2] = o[2] / o[3];
}

__device__ __forceinline__ float depth_of(const float* img, int W, int H, int x, int y) {
    x = min(max(x, 0), W - 1);  // GL_CLAMP_TO_EDGE, GL_NEAREST
    y = min(max(y, 0), H - 1);
    return img[(long long)y * W + x];
}

// ---- 1, 3, 4: sprite splats -------------------------------------------------
// The billboard of particle_sprites.vs: z = normalize(eye position),
// x = normalize(cross((0,1,0), z)), y = normalize(cross(z, x)); the FlipSquare's
// corners (+-0.5, +-0.5) scaled by 2r, texCoord = (px + 0.5, 0.5 - py).
struct Sprite {
    float c[3], xa[3], ya[3], za[3];
    int x0, x1, y0, y1;  // pixel range (inclusive)
};

__device__ __forceinline__ bool make_sprite(const Cam& cam, const float* pw, float r, int W, int H, Sprite& s) {
    const float p4[4] = {pw[0], pw[1], pw[2], 1.f};
    float e[4];
    mul4(cam.view, p4, e);
    s.c[0] = e[0]; s.c[1] = e[1]; s.c[2] = e[2];
    s.za[0] = e[0]; s.za[1] = e[1]; s.za[2] = e[2];
    normalize3(s.za);
    const float up[3] = {0.f, 1.f, 0.f};
    cross3(up, s.za, s.xa);
    normalize3(s.xa);
    cross3(s.za, s.xa, s.ya);
    normalize3(s.ya);
    // projected corners -> pixel-centre range; a sprite reaching behind the eye is skipped
    float xmin = 1e30f, xmax = -1e30f, ymin = 1e30f, ymax = -1e30f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float sx = (k & 1) ? 0.5f : -0.5f, sy = (k & 2) ? 0.5f : -0.5f;
        float q[4];
#pragma unroll
        for (int a = 0; a < 3; a++) q[a] = s.c[a] + (s.xa[a] * sx + s.ya[a] * sy) * (r * 2.f);
        q[3] = 1.f;
        float cl[4];
        mul4(cam.proj, q, cl);
        if (!(cl[3] > 0.f)) return false;
        const float wx = (cl[0] / cl[3] * 0.5f + 0.5f) * (float)W, wy = (cl[1] / cl[3] * 0.5f + 0.5f) * (float)H;
        xmin = fminf(xmin, wx); xmax = fmaxf(xmax, wx);
        ymin = fminf(ymin, wy); ymax = fmaxf(ymax, wy);
    }
    // pixel i covers centre i + 0.5 (bounds clamped before the integer conversion)
    xmin = fmaxf(xmin, -1.f); ymin = fmaxf(ymin, -1.f);
    xmax = fminf(xmax, (float)W + 1.f); ymax = fminf(ymax, (float)H + 1.f);
    s.x0 = max((int)ceilf(xmin - 0.5f), 0);
    s.x1 = min((int)floorf(xmax - 0.5f), W - 1);
    s.y0 = max((int)ceilf(ymin - 0.5f), 0);
    s.y1 = min((int)floorf(ymax - 0.5f), H - 1);
    return s.x0 <= s.x1 && s.y0 <= s.y1;
}

// Sprite coordinate of pixel (i, j): false outside the quad.  On return P is
// the eye-space point of the billboard plane under the pixel centre.
__device__ __forceinline__ bool sprite_hit(const Cam& cam, const Sprite& s, float r, int W, int H, int i, int j,
                                           float& px, float& py, float* P) {
    const float nd4[4] = {((float)i + 0.5f) / (float)W * 2.f - 1.f, ((float)j + 0.5f) / (float)H * 2.f - 1.f, -1.f,
                          1.f};
    float o[4];
    mul4(cam.proj_inv, nd4, o);
    const float d[3] = {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
    const float den = dot3(d, s.za);
    if (!(den > 0.f)) return false;
    const float t = dot3(s.c, s.za) / den;
    P[0] = d[0] * t; P[1] = d[1] * t; P[2] = d[2] * t;
    const float q[3] = {P[0] - s.c[0], P[1] - s.c[1], P[2] - s.c[2]};
    px = dot3(q, s.xa) / (r * 2.f);
    py = dot3(q, s.ya) / (r * 2.f);
    return fabsf(px) <= 0.5f && fabsf(py) <= 0.5f;
}

__device__ __forceinline__ float window_depth(const Cam& cam, const float* p, bool& inside) {
    const float q[4] = {p[0], p[1], p[2], 1.f};
    float cl[4];
    mul4(cam.proj, q, cl);
    const float z = cl[2] / cl[3];
    inside = z >= -1.f && z <= 1.f;  // near / far clipping
    return z * 0.5f + 0.5f;
}

// which: 0 all particles, 1 surface (density >= threshold), 2 spray (below).
// With `thick` set, the same fragments also add their thickness
// (particle_sprites_thickness.fs: sqrt(1 - r2) * r, GL_ONE + GL_ONE blending),
// depth-tested GL_LESS against the scene depth at the billboard plane and not
// against the fluid depth, so one pass per particle serves both splats (the
// surface and the spray passes together cover every particle once).
__global__ void k_splat_depth(const fsim_particle_gfx* parts, long long n, int which, float thr, Cam cam, float r,
                              int W, int H, unsigned* depth_bits, const float* scene, float* thick) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const fsim_particle_gfx pg = parts[k];
    if (which == 1 && pg.density < thr) return;
    if (which == 2 && !(pg.density < thr)) return;
    Sprite s;
    if (!make_sprite(cam, pg.pos, r, W, H, s)) return;
    for (int j = s.y0; j <= s.y1; j++)
        for (int i = s.x0; i <= s.x1; i++) {
            float px, py, P[3];
            if (!sprite_hit(cam, s, r, W, H, i, j, px, py, P)) continue;
            bool inside;
            const float zq = window_depth(cam, P, inside);
            if (!inside) continue;
            // particle_sprites_depth.fs
            const float nx = px * 2.f, ny = -py * 2.f;  // texCoord * 2 - 1
            const float r2 = nx * nx + ny * ny;
            if (r2 > 1.f) continue;
            const long long pix = (long long)j * W + i;
            if (thick && zq < (scene ? scene[pix] : 1.f)) atomicAdd(&thick[pix], sqrtf(1.f - r2) * r);
            const float nz = -sqrtf(1.f - r2);
            float nrm[3];
#pragma unroll
            for (int a = 0; a < 3; a++) nrm[a] = s.xa[a] * nx + s.ya[a] * ny + s.za[a] * nz;
            normalize3(nrm);
            float pp[3];
#pragma unroll
            for (int a = 0; a < 3; a++) pp[a] = s.c[a] + nrm[a] * r;
            bool in2;
            float z = window_depth(cam, pp, in2);
            z = fminf(fmaxf(z, 0.f), 1.f);  // gl_FragDepth is clamped to the depth range
            atomicMin(&depth_bits[pix], __float_as_uint(z));  // z >= 0: bits order as floats
        }
}

__global__ void k_fill(float* p, long long n, float v) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = v;
}

__global__ void k_fill4(float4* p, long long n, float4 v) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = v;
}

// ---- 2, 4: separable blurs -----------------------------------------------------
// Kernel extent from the world-space smoothing size projected at the pixel
// (gaussian.fs / bilateral.fs / gaussian_thickness.fs).
__device__ __forceinline__ float screen_extent(const Cam& cam, const float* eye, float size, int axis, float u,
                                               float v) {
    float q[4] = {eye[0], eye[1], eye[2], 1.f};
    q[axis] = q[axis] + size * 0.5f;
    float o[4];
    mul4(cam.proj, q, o);
    return axis == 0 ? o[0] / o[3] * 0.5f + 0.5f - u : o[1] / o[3] * 0.5f + 0.5f - v;
}

// mode 0: Gaussian depth, 1: bilateral depth, 2: Gaussian thickness (src = thickness, dsrc = depth)
__global__ void k_blur(int mode, int axis, const float* src, const float* dsrc, float* dst, int W, int H, Cam cam,
                       float size, float blur_scale, float falloff) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)W * H) return;
    const int x = (int)(id % W), y = (int)(id / W);
    const float cur = dsrc[id];
    if (cur == 1.f) {
        dst[id] = mode == 2 ? 0.f : 1.f;  // discarded: the cleared value stays
        return;
    }
    const float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
    float eye[3];
    uv_to_eye(cam, u, v, cur, eye);
    const int tex = axis == 0 ? W : H;
    const float ext = screen_extent(cam, eye, size, axis, u, v);
    float acc = 0.f, wsum = 0.f;
    if (mode == 1) {
        int R = (int)(ext * (float)tex);
        R = R > 35 ? 35 : (R < 1 ? 1 : R);
        for (int p = -R; p <= R; p++) {
            const float s = axis == 0 ? depth_of(src, W, H, x + p, y) : depth_of(src, W, H, x, y + p);
            if (s < 1.f) {
                const float rr = (float)p * blur_scale;
                const float w = expf(-rr * rr);
                const float r2 = (s - cur) * falloff;
                const float g = expf(-r2 * r2);
                acc = acc + s * w * g;
                wsum = wsum + w * g;
            }
        }
        dst[id] = wsum == 0.f ? 1.f : acc / wsum;
        return;
    }
    int ks = (int)(ext * (float)tex) * 2 + 1;
    ks = ks > 51 ? 51 : (ks < 3 ? 3 : ks);
    const float sd = (float)(ks - 1) / 6.f;
    const float sd2 = sd * sd;
    const int R = ks / 2;
    for (int p = -R; p <= R; p++) {
        const float s = axis == 0 ? depth_of(src, W, H, x + p, y) : depth_of(src, W, H, x, y + p);
        if (mode == 2 || s < 1.f) {
            const float w = expf((float)(-p * p) / sd2 * 0.5f);
            wsum = wsum + w;
            acc = acc + s * w;
        }
    }
    dst[id] = acc / wsum;
}

// ---- 5: normals (normal_depth.fs) ---------------------------------------------
__device__ __forceinline__ void eye_at(const Cam& cam, const float* depth, int W, int H, int x, int y, float* e) {
    const int cx = min(max(x, 0), W - 1), cy = min(max(y, 0), H - 1);
    // texCoord + texel offset, sampled with GL_NEAREST and CLAMP_TO_EDGE: the
    // coordinate is the unclamped one, the value the clamped texel's
    const float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
    uv_to_eye(cam, u, v, depth[(long long)cy * W + cx], e);
}

__global__ void k_normals(const float* depth, float4* nd, int W, int H, Cam cam) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)W * H) return;
    const int x = (int)(id % W), y = (int)(id / W);
    const float d = depth[id];
    if (d == 1.f) {
        nd[id] = make_float4(0.f, 0.f, 0.f, 1.f);
        return;
    }
    float p[3], a[3], b[3], ddx[3], ddx2[3], ddy[3], ddy2[3];
    eye_at(cam, depth, W, H, x, y, p);
    eye_at(cam, depth, W, H, x + 1, y, a);
    eye_at(cam, depth, W, H, x - 1, y, b);
#pragma unroll
    for (int k = 0; k < 3; k++) { ddx[k] = a[k] - p[k]; ddx2[k] = p[k] - b[k]; }
    if (fabsf(ddx[2]) > fabsf(ddx2[2])) { ddx[0] = ddx2[0]; ddx[1] = ddx2[1]; ddx[2] = ddx2[2]; }
    eye_at(cam, depth, W, H, x, y + 1, a);
    eye_at(cam, depth, W, H, x, y - 1, b);
#pragma unroll
    for (int k = 0; k < 3; k++) { ddy[k] = a[k] - p[k]; ddy2[k] = p[k] - b[k]; }
    if (fabsf(ddy2[2]) < fabsf(ddy[2])) { ddy[0] = ddy2[0]; ddy[1] = ddy2[1]; ddy[2] = ddy2[2]; }
    float n[3];
    cross3(ddx, ddy, n);
    normalize3(n);
    const float n4[4] = {n[0], n[1], n[2], 0.f};
    float w[4];
    mul4(cam.view_inv, n4, w);
    nd[id] = make_float4(w[0], w[1], w[2], d);
}

// ---- 6: shading (shadedDepth.fs) ------------------------------------------------
// Classic 3D Perlin noise in the form of Gustavson's shader: lattice hashes by
// the permutation polynomial (34 x + 10) x mod 289, gradients on the surface
// of an octahedron from the hash, quintic fade, scaled by 2.2.
__device__ __forceinline__ float mod289(float x) { return x - floorf(x * (1.f / 289.f)) * 289.f; }
__device__ __forceinline__ float permute(float x) { return mod289((x * 34.f + 10.f) * x); }
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.f - t) + b * t; }

__device__ float perlin(float X, float Y, float Z) {
    const float i0[3] = {mod289(floorf(X)), mod289(floorf(Y)), mod289(floorf(Z))};
    const float i1[3] = {mod289(floorf(X) + 1.f), mod289(floorf(Y) + 1.f), mod289(floorf(Z) + 1.f)};
    const float f0[3] = {fractf(X), fractf(Y), fractf(Z)};
    const float f1[3] = {f0[0] - 1.f, f0[1] - 1.f, f0[2] - 1.f};
    float n[2][4];  // [z corner][xy corner: (0,0) (1,0) (0,1) (1,1)]
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int cx = c & 1, cy = c >> 1;
        const float hxy = permute(permute(cx ? i1[0] : i0[0]) + (cy ? i1[1] : i0[1]));
#pragma unroll
        for (int cz = 0; cz < 2; cz++) {
            const float h = permute(hxy + (cz ? i1[2] : i0[2]));
            float gx = h * (1.f / 7.f);
            float gy = fractf(floorf(gx) * (1.f / 7.f)) - 0.5f;
            gx = fractf(gx);
            const float gz = 0.5f - fabsf(gx) - fabsf(gy);
            const float sz = gz <= 0.f ? 1.f : 0.f;  // step(gz, 0)
            gx = gx - sz * ((gx < 0.f ? 0.f : 1.f) - 0.5f);
            gy = gy - sz * ((gy < 0.f ? 0.f : 1.f) - 0.5f);
            const float norm = 1.79284291400159f - 0.85373472095314f * (gx * gx + gy * gy + gz * gz);
            n[cz][c] = (gx * norm) * (cx ? f1[0] : f0[0]) + (gy * norm) * (cy ? f1[1] : f0[1]) +
                       (gz * norm) * (cz ? f1[2] : f0[2]);
        }
    }
    const float fx = fade(f0[0]), fy = fade(f0[1]), fz = fade(f0[2]);
    float nz[4];
#pragma unroll
    for (int c = 0; c < 4; c++) nz[c] = mixf(n[0][c], n[1][c], fz);
    const float ny0 = mixf(nz[0], nz[2], fy), ny1 = mixf(nz[1], nz[3], fy);
    return 2.2f * mixf(ny0, ny1, fx);
}

struct ShadeArgs {
    Cam cam;
    int W, H;
    const float4* nd;
    const float* thick;
    const float* scene;
    float4* color;
    float diffuse[4], specular[3], shininess;
    int transparency_enabled;
    float transparency;
    int noise_enabled;
    float noise_scale, noise_strength, noise_offset;
    int nl;
    fsim_light lights[FSIM_RENDER_MAX_LIGHTS];
    float bg[4];
};

__device__ __forceinline__ void world_at(const ShadeArgs& a, int x, int y, float* w, float* nrm) {
    const int cx = min(max(x, 0), a.W - 1), cy = min(max(y, 0), a.H - 1);
    const float4 t = a.nd[(long long)cy * a.W + cx];
    const float u = ((float)x + 0.5f) / (float)a.W, v = ((float)y + 0.5f) / (float)a.H;
    float e[3];
    uv_to_eye(a.cam, u, v, t.w, e);
    const float e4[4] = {e[0], e[1], e[2], 1.f};
    float o[4];
    mul4(a.cam.view_inv, e4, o);
    w[0] = o[0]; w[1] = o[1]; w[2] = o[2];
    nrm[0] = t.x; nrm[1] = t.y; nrm[2] = t.z;
}

// getNoiseOffsetWorldSpacePos
__device__ __forceinline__ void noisy_pos(const ShadeArgs& a, int x, int y, float* out) {
    float w[3], n[3];
    world_at(a, x, y, w, n);
    const float px = w[0] * a.noise_scale, py = w[1] * a.noise_scale, pz = w[2] * a.noise_scale;
    const float noise =
        perlin(px + a.noise_offset, py, pz) + perlin(-px + a.noise_offset, py + a.noise_offset, pz);
#pragma unroll
    for (int k = 0; k < 3; k++) out[k] = w[k] + n[k] * noise;
}

__device__ void shade_light(const float* wp, const float* nrm_in, const float* view, const fsim_light& L,
                            const float* mat, const float* spec, float shininess, float* acc) {
    float f2l[3];
#pragma unroll
    for (int k = 0; k < 3; k++) f2l[k] = L.position[k] - wp[k] * L.position[3];
    float ld[3] = {f2l[0], f2l[1], f2l[2]};
    normalize3(ld);
    float n[3] = {nrm_in[0], nrm_in[1], nrm_in[2]};
    if (dot3(n, view) < 0.f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
    const float lc = dot3(ld, n);
    if (lc < 0.f) return;
    float d2 = sqrtf(dot3(f2l, f2l));
    d2 = d2 * d2;
    float hw[3] = {view[0] + ld[0], view[1] + ld[1], view[2] + ld[2]};
    normalize3(hw);
    float shine = dot3(hw, n);
    if (shine < 0.f) shine = 0.f;
    const float sp = powf(shine, shininess);
#pragma unroll
    for (int k = 0; k < 3; k++) acc[k] = acc[k] + L.power_density[k] * (mat[k] * lc + spec[k] * sp) / d2;
}

__global__ void k_shade(const ShadeArgs a) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)a.W * a.H) return;
    const int x = (int)(id % a.W), y = (int)(id / a.W);
    const float4 t = a.nd[id];
    const float4 bg = make_float4(a.bg[0], a.bg[1], a.bg[2], a.bg[3]);
    if (t.w == 1.f || (a.scene && !(t.w < a.scene[id]))) {
        a.color[id] = bg;
        return;
    }
    float wp[3], n[3];
    world_at(a, x, y, wp, n);
    if (a.noise_enabled) {
        float p[3], q[3], ddx[3], ddx2[3], ddy[3], ddy2[3];
        noisy_pos(a, x, y, p);
        noisy_pos(a, x + 1, y, q);
#pragma unroll
        for (int k = 0; k < 3; k++) ddx[k] = q[k] - p[k];
        noisy_pos(a, x - 1, y, q);
#pragma unroll
        for (int k = 0; k < 3; k++) ddx2[k] = p[k] - q[k];
        if (fabsf(ddx[2]) > fabsf(ddx2[2])) { ddx[0] = ddx2[0]; ddx[1] = ddx2[1]; ddx[2] = ddx2[2]; }
        noisy_pos(a, x, y + 1, q);
#pragma unroll
        for (int k = 0; k < 3; k++) ddy[k] = q[k] - p[k];
        noisy_pos(a, x, y - 1, q);
#pragma unroll
        for (int k = 0; k < 3; k++) ddy2[k] = p[k] - q[k];
        if (fabsf(ddy2[2]) < fabsf(ddy[2])) { ddy[0] = ddy2[0]; ddy[1] = ddy2[1]; ddy[2] = ddy2[2]; }
        float nn[3];
        cross3(ddx, ddy, nn);
        normalize3(nn);
        const float s = a.noise_strength;
#pragma unroll
        for (int k = 0; k < 3; k++) n[k] = n[k] * (1.f - s) + nn[k] * s;
        normalize3(n);
    }
    float c[4] = {0.f, 0.f, 0.f, a.diffuse[3]};
    if (a.transparency_enabled) c[3] = expf(-a.transparency * a.thick[id]);
    float view[3] = {a.cam.pos[0] - wp[0], a.cam.pos[1] - wp[1], a.cam.pos[2] - wp[2]};
    normalize3(view);
    for (int l = 0; l < a.nl; l++) shade_light(wp, n, view, a.lights[l], a.diffuse, a.specular, a.shininess, c);
    if (a.transparency_enabled) {
        // glBlendFunc(GL_ONE_MINUS_SRC_ALPHA, GL_SRC_ALPHA) over the background
        const float al = c[3];
        a.color[id] = make_float4(c[0] * (1.f - al) + bg.x * al, c[1] * (1.f - al) + bg.y * al,
                                  c[2] * (1.f - al) + bg.z * al, c[3] * (1.f - al) + bg.w * al);
    } else {
        a.color[id] = make_float4(c[0], c[1], c[2], c[3]);
    }
}

// ---- host helpers ----------------------------------------------------------------
inline unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

void to_cam(const fsim_camera& c, Cam& k) {
    std::memcpy(k.view.m, c.view, sizeof(k.view.m));
    std::memcpy(k.view_inv.m, c.view_inv, sizeof(k.view_inv.m));
    std::memcpy(k.proj.m, c.proj, sizeof(k.proj.m));
    std::memcpy(k.proj_inv.m, c.proj_inv, sizeof(k.proj_inv.m));
    std::memcpy(k.pos, c.position, sizeof(k.pos));
}

// general 4x4 inverse (cofactor expansion), column-major
bool invert4(const double* m, double* inv) {
    double t[16];
    t[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
           m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    t[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
           m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    t[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
           m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    t[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
            m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    t[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
           m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    t[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
           m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    t[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
           m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    t[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
            m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    t[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
           m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    t[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
           m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    t[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
            m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    t[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
            m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    t[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
           m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    t[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
           m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    t[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
            m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    t[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
            m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * t[0] + m[1] * t[4] + m[2] * t[8] + m[3] * t[12];
    if (det == 0.0) return false;
    for (int i = 0; i < 16; i++) inv[i] = t[i] / det;
    return true;
}

int fail(fsim_renderer* r, int code, const std::string& msg) {
    if (r) r->err = msg;
    return code;
}

int ensure_parts(fsim_renderer* r, long long n) {
    if (n <= r->parts_cap) return FSIM_OK;
    cudaFree(r->parts);
    r->parts = nullptr;
    r->parts_cap = 0;
    const long long cap = n + n / 4 + 1024;
    if (cudaMalloc(&r->parts, (size_t)cap * sizeof(fsim_particle_gfx)) != cudaSuccess) {
        cudaGetLastError();
        return fail(r, FSIM_E_OOM, "particle staging buffer");
    }
    r->parts_cap = cap;
    return FSIM_OK;
}

}  // namespace

extern "C" {

void fsim_render_default_params(fsim_render_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->particle_radius = 1.f / 1024.f;
    p->particle_color[0] = 0.f; p->particle_color[1] = 0.4f; p->particle_color[2] = 0.95f;
    p->specular_color[0] = p->specular_color[1] = p->specular_color[2] = 1.2f;
    p->shininess = 80.f;
    p->bilateral_filter = 0;
    p->smoothing_size = 2.4f;
    p->blur_scale = 0.083f;
    p->blur_depth_falloff = 1100.f;
    p->spray_enabled = 1;
    p->spray_density_threshold = 1.2f;
    p->transparency_enabled = 1;
    p->transparency_blur_size = 2.4f;
    p->transparency = 1.334f;
    p->noise_enabled = 1;
    p->noise_scale = 0.956f;
    p->noise_strength = 0.123f;
    p->noise_offset = 0.f;
    const float lp[4][4] = {{50, 50, 50, 1}, {50, 50, -50, 1}, {-50, 50, -50, 1}, {-50, 50, 50, 1}};
    const float pd[4][3] = {{1000, 2000, 2000}, {2000, 1000, 2000}, {2000, 2000, 1000}, {2000, 2000, 2000}};
    p->num_lights = 4;
    for (int l = 0; l < 4; l++) {
        std::memcpy(p->lights[l].position, lp[l], sizeof(lp[l]));
        std::memcpy(p->lights[l].power_density, pd[l], sizeof(pd[l]));
    }
    p->background[0] = p->background[1] = p->background[2] = 0.f;
    p->background[3] = 1.f;
}

void fsim_render_camera(fsim_camera* cam, const double eye[3], double yaw_deg, double pitch_deg, double fov_deg,
                        double aspect, double z_near, double z_far) {
    if (!cam || !eye) return;
    const double kPi = 3.14159265358979323846;
    const double yaw = yaw_deg * kPi / 180.0, pitch = pitch_deg * kPi / 180.0;
    double f[3] = {std::cos(yaw) * std::cos(pitch), std::sin(pitch), std::sin(yaw) * std::cos(pitch)};
    auto norm = [](double* v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] /= l; v[1] /= l; v[2] /= l;
    };
    auto cross = [](const double* a, const double* b, double* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    norm(f);
    // Camera3D::updateViewMatrix: right = cross(front, +y), up = cross(right, front)
    const double yup[3] = {0, 1, 0};
    double right[3], up[3];
    cross(f, yup, right);
    norm(right);
    cross(right, f, up);
    norm(up);
    // lookAt(eye, eye + f, up), right-handed
    double s[3], u[3];
    cross(f, up, s);
    norm(s);
    cross(s, f, u);
    double V[16] = {0};
    V[0] = s[0]; V[4] = s[1]; V[8] = s[2];
    V[1] = u[0]; V[5] = u[1]; V[9] = u[2];
    V[2] = -f[0]; V[6] = -f[1]; V[10] = -f[2];
    V[12] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    V[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    V[14] = f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2];
    V[15] = 1;
    // perspective(fov, aspect, near, far), OpenGL clip depth [-1, 1]
    const double th = std::tan(fov_deg * kPi / 180.0 / 2.0);
    double P[16] = {0};
    P[0] = 1.0 / (aspect * th);
    P[5] = 1.0 / th;
    P[10] = -(z_far + z_near) / (z_far - z_near);
    P[11] = -1.0;
    P[14] = -(2.0 * z_far * z_near) / (z_far - z_near);
    double Vi[16], Pi[16];
    invert4(V, Vi);
    invert4(P, Pi);
    for (int i = 0; i < 16; i++) {
        cam->view[i] = (float)V[i];
        cam->view_inv[i] = (float)Vi[i];
        cam->proj[i] = (float)P[i];
        cam->proj_inv[i] = (float)Pi[i];
    }
    cam->position[0] = (float)eye[0];
    cam->position[1] = (float)eye[1];
    cam->position[2] = (float)eye[2];
    cam->position[3] = 1.f;
}

int fsim_render_create(int width, int height, fsim_renderer** out) {
    if (!out || width <= 0 || height <= 0 || (long long)width * height > (1ll << 28)) return FSIM_E_INVALID;
    *out = nullptr;
    fsim_renderer* r = new (std::nothrow) fsim_renderer();
    if (!r) return FSIM_E_OOM;
    r->W = width;
    r->H = height;
    const size_t np = (size_t)width * height;
    bool ok = cudaStreamCreateWithFlags(&r->own, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&r->raw, np * 4) == cudaSuccess && cudaMalloc(&r->depth, np * 4) == cudaSuccess &&
              cudaMalloc(&r->tmp, np * 4) == cudaSuccess && cudaMalloc(&r->thick, np * 4) == cudaSuccess &&
              cudaMalloc(&r->ttmp, np * 4) == cudaSuccess && cudaMalloc(&r->nd, np * 16) == cudaSuccess &&
              cudaMalloc(&r->color, np * 16) == cudaSuccess && cudaEventCreate(&r->ev0) == cudaSuccess &&
              cudaEventCreate(&r->ev1) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fsim_render_destroy(r);
        return FSIM_E_OOM;
    }
    *out = r;
    return FSIM_OK;
}

int fsim_render_destroy(fsim_renderer* r) {
    if (!r) return FSIM_OK;
    if (r->own) cudaStreamSynchronize(r->own);
    if (r->last) cudaStreamSynchronize(r->last);
    cudaFree(r->raw); cudaFree(r->depth); cudaFree(r->tmp); cudaFree(r->thick); cudaFree(r->ttmp);
    cudaFree(r->nd); cudaFree(r->color); cudaFree(r->parts);
    if (r->ev0) cudaEventDestroy(r->ev0);
    if (r->ev1) cudaEventDestroy(r->ev1);
    if (r->own) cudaStreamDestroy(r->own);
    delete r;
    return FSIM_OK;
}

const char* fsim_render_last_error(fsim_renderer* r) { return r ? r->err.c_str() : "null renderer"; }

int fsim_render_frame(fsim_renderer* r, const fsim_particle_gfx* particles, int64_t n, int where,
                      const fsim_camera* cam, const fsim_render_params* prm, const float* scene_depth,
                      void* stream) {
    if (!r || !cam || !prm || n < 0 || (n > 0 && !particles)) return fail(r, FSIM_E_INVALID, "invalid argument");
    if (prm->num_lights < 0 || prm->num_lights > FSIM_RENDER_MAX_LIGHTS || !(prm->particle_radius > 0.f))
        return fail(r, FSIM_E_INVALID, "num_lights or particle_radius");
    cudaStream_t s = stream ? (cudaStream_t)stream : r->own;
    r->last = s;
    const fsim_particle_gfx* dp = particles;
    if (where == FSIM_HOST && n > 0) {
        int rc = ensure_parts(r, n);
        if (rc) return rc;
        if (cudaMemcpyAsync(r->parts, particles, (size_t)n * sizeof(fsim_particle_gfx), cudaMemcpyHostToDevice,
                            s) != cudaSuccess)
            return fail(r, FSIM_E_CUDA, "particle upload");
        dp = r->parts;
    }
    Cam k;
    to_cam(*cam, k);
    const int W = r->W, H = r->H;
    const long long np = (long long)W * H;
    const float rad = prm->particle_radius;
    int L = 0;
    cudaEventRecord(r->ev0, s);
    // 1. surface sprites into the cleared depth buffer, with their thickness
    //    (the thickness of all particles accumulates over passes 1 and 3)
    float* thick = prm->transparency_enabled ? r->thick : nullptr;
    k_fill<<<nblk(np), 256, 0, s>>>(r->raw, np, 1.f);
    k_fill<<<nblk(np), 256, 0, s>>>(r->thick, np, 0.f);
    L += 2;
    if (n > 0) {
        k_splat_depth<<<nblk(n), 256, 0, s>>>(dp, n, prm->spray_enabled ? 1 : 0, prm->spray_density_threshold, k,
                                              rad, W, H, reinterpret_cast<unsigned*>(r->raw), scene_depth, thick);
        L++;
    }
    // 2. smoothing, x into tmp then y into depth
    const int mode = prm->bilateral_filter ? 1 : 0;
    k_blur<<<nblk(np), 256, 0, s>>>(mode, 0, r->raw, r->raw, r->tmp, W, H, k, prm->smoothing_size, prm->blur_scale,
                                   prm->blur_depth_falloff);
    k_blur<<<nblk(np), 256, 0, s>>>(mode, 1, r->tmp, r->tmp, r->depth, W, H, k, prm->smoothing_size,
                                   prm->blur_scale, prm->blur_depth_falloff);
    L += 2;
    // 3. spray on top of the smoothed surface
    if (prm->spray_enabled && n > 0) {
        k_splat_depth<<<nblk(n), 256, 0, s>>>(dp, n, 2, prm->spray_density_threshold, k, rad, W, H,
                                              reinterpret_cast<unsigned*>(r->depth), scene_depth, thick);
        L++;
    }
    // 4. thickness blurred x then y
    if (prm->transparency_enabled) {
        k_blur<<<nblk(np), 256, 0, s>>>(2, 0, r->thick, r->depth, r->ttmp, W, H, k, prm->transparency_blur_size,
                                       0.f, 0.f);
        k_blur<<<nblk(np), 256, 0, s>>>(2, 1, r->ttmp, r->depth, r->thick, W, H, k, prm->transparency_blur_size,
                                       0.f, 0.f);
        L += 2;
    }
    // 5. normals
    k_normals<<<nblk(np), 256, 0, s>>>(r->depth, r->nd, W, H, k);
    L++;
    // 6. shading and composite
    ShadeArgs a;
    a.cam = k;
    a.W = W;
    a.H = H;
    a.nd = r->nd;
    a.thick = r->thick;
    a.scene = scene_depth;
    a.color = r->color;
    for (int q = 0; q < 3; q++) {
        a.diffuse[q] = prm->particle_color[q];
        a.specular[q] = prm->specular_color[q];
    }
    a.diffuse[3] = 1.f;
    a.shininess = prm->shininess;
    a.transparency_enabled = prm->transparency_enabled;
    a.transparency = prm->transparency;
    a.noise_enabled = prm->noise_enabled;
    a.noise_scale = prm->noise_scale;
    a.noise_strength = prm->noise_strength;
    a.noise_offset = prm->noise_offset;
    a.nl = prm->num_lights;
    std::memcpy(a.lights, prm->lights, sizeof(a.lights));
    std::memcpy(a.bg, prm->background, sizeof(a.bg));
    k_shade<<<nblk(np), 256, 0, s>>>(a);
    L++;
    cudaEventRecord(r->ev1, s);
    r->timed = true;
    r->launches = L;
    if (cudaGetLastError() != cudaSuccess) return fail(r, FSIM_E_CUDA, "render kernel launch failed");
    return FSIM_OK;
}

int fsim_render_read(fsim_renderer* r, int image, void* dst, int where) {
    if (!r || !dst) return FSIM_E_INVALID;
    const size_t np = (size_t)r->W * r->H;
    const void* src = nullptr;
    size_t bytes = np * 4;
    switch (image) {
        case FSIM_IMG_COLOR: src = r->color; bytes = np * 16; break;
        case FSIM_IMG_DEPTH: src = r->depth; break;
        case FSIM_IMG_THICKNESS: src = r->thick; break;
        case FSIM_IMG_NORMAL_DEPTH: src = r->nd; bytes = np * 16; break;
        case FSIM_IMG_RAW_DEPTH: src = r->raw; break;
        default: return fail(r, FSIM_E_INVALID, "unknown image");
    }
    cudaStream_t s = r->last ? r->last : r->own;
    if (cudaMemcpyAsync(dst, src, bytes, where == FSIM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                        s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(r, FSIM_E_CUDA, "image copy");
    return FSIM_OK;
}

int fsim_render_stats(fsim_renderer* r, float* ms, int* launches) {
    if (!r) return FSIM_E_INVALID;
    if (launches) *launches = r->launches;
    if (ms) {
        *ms = 0.f;
        if (r->timed) {
            if (cudaEventSynchronize(r->ev1) != cudaSuccess ||
                cudaEventElapsedTime(ms, r->ev0, r->ev1) != cudaSuccess) {
                cudaGetLastError();
                return fail(r, FSIM_E_CUDA, "frame timing");
            }
        }
    }
    return FSIM_OK;
}

int fsim_render_ctx(fsim_renderer* r, fsim_ctx* ctx, const fsim_camera* cam, const fsim_render_params* params,
                    const float* scene_depth) {
    if (!r || !ctx) return FSIM_E_INVALID;
    int64_t n = 0;
    int rc = fsim_num_particles(ctx, &n);
    if (rc) return fail(r, rc, "fsim_num_particles");
    if ((rc = ensure_parts(r, n))) return rc;
    int64_t got = 0;
    if (n > 0 && (rc = fsim_fill_gfx(ctx, r->parts, r->parts_cap, &got, FSIM_DEVICE)))
        return fail(r, rc, std::string("fsim_fill_gfx: ") + fsim_last_error(ctx));
    return fsim_render_frame(r, r->parts, got, FSIM_DEVICE, cam, params, scene_depth, fsim_stream(ctx));
}

}  // extern "C"
