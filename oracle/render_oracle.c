/* render_oracle.c -- TEST INFRASTRUCTURE ONLY: the CPU restatement of the
 * reference's screen-space fluid shaders that the CUDA renderer
 * (fluid_simulator_gb300/csrc/k_render.cu) is checked against.  Nothing in the
 * library calls it.
 *
 * The reference renders with OpenGL (FluidSurfaceGfx::render,
 * src/Application/gfx/gfx3D/fluidSurfaceGfx.cpp:81-204); no OpenGL exists where
 * this runs, so the reference itself cannot produce images here and parity of
 * the renderer is pinned to this restatement of the shader sources only:
 *   src/shaders/particle_sprites.vs:24-51 (billboard), particle_sprites_depth.fs:20-40,
 *   gaussian.fs:18-89, bilateral.fs:20-98, particle_sprites_thickness.fs:20-28,
 *   gaussian_thickness.fs:20-87, normal_depth.fs:18-53, shadedDepth.fs:38-224
 *   (uvToEye, shade, getNoiseOffsetWorldSpacePos, getNormalWithNoise, main, cnoise).
 * Rasterisation is restated as: the pixel centres inside the projected
 * billboard, each with the sprite coordinate where its eye ray meets the
 * billboard plane (perspective-correct texCoord); depth test GL_LESS, clear
 * 1.0; textures GL_NEAREST with GL_CLAMP_TO_EDGE; blending as in render().
 * FP32 throughout, like the shaders; built with -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/fsim_render.h"

typedef struct {
    const float *view, *view_inv, *proj, *proj_inv, *pos;
} cam_t;

static void mul4(const float *M, const float v[4], float o[4]) {
    for (int r = 0; r < 4; r++) {
        float s = M[r] * v[0];
        s = s + M[4 + r] * v[1];
        s = s + M[8 + r] * v[2];
        s = s + M[12 + r] * v[3];
        o[r] = s;
    }
}

static float dot3(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void cross3(const float *a, const float *b, float *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static void normalize3(float *v) {
    float l = sqrtf(dot3(v, v));
    if (l > 0.f) {
        v[0] = v[0] / l;
        v[1] = v[1] / l;
        v[2] = v[2] / l;
    }
}

static void uv_to_eye(const cam_t *c, float u, float v, float d, float *e) {
    float ndc[4] = {u * 2.f - 1.f, v * 2.f - 1.f, d * 2.f - 1.f, 1.f}, o[4];
    mul4(c->proj_inv, ndc, o);
    e[0] = o[0] / o[3];
    e[1] = o[1] / o[3];
    e[2] = o[2] / o[3];
}

static int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

static float tex(const float *img, int W, int H, int x, int y) {
    return img[(int64_t)clampi(y, 0, H - 1) * W + clampi(x, 0, W - 1)];
}

/* ---- sprites --------------------------------------------------------- */
typedef struct {
    float c[3], xa[3], ya[3], za[3];
    int x0, x1, y0, y1;
} sprite;

static int make_sprite(const cam_t *cam, const float *pw, float r, int W, int H, sprite *s) {
    float p4[4] = {pw[0], pw[1], pw[2], 1.f}, e[4];
    mul4(cam->view, p4, e);
    for (int a = 0; a < 3; a++) s->c[a] = s->za[a] = e[a];
    normalize3(s->za);
    const float up[3] = {0.f, 1.f, 0.f};
    cross3(up, s->za, s->xa);
    normalize3(s->xa);
    cross3(s->za, s->xa, s->ya);
    normalize3(s->ya);
    float xmin = 1e30f, xmax = -1e30f, ymin = 1e30f, ymax = -1e30f;
    for (int k = 0; k < 4; k++) {
        float sx = (k & 1) ? 0.5f : -0.5f, sy = (k & 2) ? 0.5f : -0.5f, q[4], cl[4];
        for (int a = 0; a < 3; a++) q[a] = s->c[a] + (s->xa[a] * sx + s->ya[a] * sy) * (r * 2.f);
        q[3] = 1.f;
        mul4(cam->proj, q, cl);
        if (!(cl[3] > 0.f)) return 0;
        float wx = (cl[0] / cl[3] * 0.5f + 0.5f) * (float)W, wy = (cl[1] / cl[3] * 0.5f + 0.5f) * (float)H;
        xmin = fminf(xmin, wx); xmax = fmaxf(xmax, wx);
        ymin = fminf(ymin, wy); ymax = fmaxf(ymax, wy);
    }
    xmin = fmaxf(xmin, -1.f); ymin = fmaxf(ymin, -1.f);
    xmax = fminf(xmax, (float)W + 1.f); ymax = fminf(ymax, (float)H + 1.f);
    s->x0 = (int)ceilf(xmin - 0.5f); if (s->x0 < 0) s->x0 = 0;
    s->x1 = (int)floorf(xmax - 0.5f); if (s->x1 > W - 1) s->x1 = W - 1;
    s->y0 = (int)ceilf(ymin - 0.5f); if (s->y0 < 0) s->y0 = 0;
    s->y1 = (int)floorf(ymax - 0.5f); if (s->y1 > H - 1) s->y1 = H - 1;
    return s->x0 <= s->x1 && s->y0 <= s->y1;
}

static int sprite_hit(const cam_t *cam, const sprite *s, float r, int W, int H, int i, int j, float *px, float *py,
                      float *P) {
    float nd4[4] = {((float)i + 0.5f) / (float)W * 2.f - 1.f, ((float)j + 0.5f) / (float)H * 2.f - 1.f, -1.f, 1.f};
    float o[4];
    mul4(cam->proj_inv, nd4, o);
    float d[3] = {o[0] / o[3], o[1] / o[3], o[2] / o[3]};
    float den = dot3(d, s->za);
    if (!(den > 0.f)) return 0;
    float t = dot3(s->c, s->za) / den;
    P[0] = d[0] * t; P[1] = d[1] * t; P[2] = d[2] * t;
    float q[3] = {P[0] - s->c[0], P[1] - s->c[1], P[2] - s->c[2]};
    *px = dot3(q, s->xa) / (r * 2.f);
    *py = dot3(q, s->ya) / (r * 2.f);
    return fabsf(*px) <= 0.5f && fabsf(*py) <= 0.5f;
}

static float window_depth(const cam_t *cam, const float *p, int *inside) {
    float q[4] = {p[0], p[1], p[2], 1.f}, cl[4];
    mul4(cam->proj, q, cl);
    float z = cl[2] / cl[3];
    *inside = z >= -1.f && z <= 1.f;
    return z * 0.5f + 0.5f;
}

/* which: 0 all, 1 surface (density >= thr), 2 spray (density < thr) */
static void splat_depth(const fsim_particle_gfx *pt, int64_t n, int which, float thr, const cam_t *cam, float r,
                        int W, int H, float *depth) {
    for (int64_t k = 0; k < n; k++) {
        if (which == 1 && pt[k].density < thr) continue;
        if (which == 2 && !(pt[k].density < thr)) continue;
        sprite s;
        if (!make_sprite(cam, pt[k].pos, r, W, H, &s)) continue;
        for (int j = s.y0; j <= s.y1; j++)
            for (int i = s.x0; i <= s.x1; i++) {
                float px, py, P[3];
                int inside, in2;
                if (!sprite_hit(cam, &s, r, W, H, i, j, &px, &py, P)) continue;
                window_depth(cam, P, &inside);
                if (!inside) continue;
                float nx = px * 2.f, ny = -py * 2.f, r2 = nx * nx + ny * ny;
                if (r2 > 1.f) continue;
                float nz = -sqrtf(1.f - r2), nrm[3], pp[3];
                for (int a = 0; a < 3; a++) nrm[a] = s.xa[a] * nx + s.ya[a] * ny + s.za[a] * nz;
                normalize3(nrm);
                for (int a = 0; a < 3; a++) pp[a] = s.c[a] + nrm[a] * r;
                float z = window_depth(cam, pp, &in2);
                z = fminf(fmaxf(z, 0.f), 1.f);
                float *dst = &depth[(int64_t)j * W + i];
                if (z < *dst) *dst = z;
            }
    }
}

static void splat_thickness(const fsim_particle_gfx *pt, int64_t n, const cam_t *cam, float r, int W, int H,
                            const float *scene, float *thick) {
    for (int64_t k = 0; k < n; k++) {
        sprite s;
        if (!make_sprite(cam, pt[k].pos, r, W, H, &s)) continue;
        for (int j = s.y0; j <= s.y1; j++)
            for (int i = s.x0; i <= s.x1; i++) {
                float px, py, P[3];
                int inside;
                if (!sprite_hit(cam, &s, r, W, H, i, j, &px, &py, P)) continue;
                float z = window_depth(cam, P, &inside);
                if (!inside) continue;
                float sd = scene ? scene[(int64_t)j * W + i] : 1.f;
                if (!(z < sd)) continue;
                float nx = px * 2.f, ny = -py * 2.f, r2 = nx * nx + ny * ny;
                if (r2 > 1.f) continue;
                thick[(int64_t)j * W + i] += sqrtf(1.f - r2) * r;
            }
    }
}

/* ---- blurs ----------------------------------------------------------- */
static float screen_extent(const cam_t *cam, const float *eye, float size, int axis, float u, float v) {
    float q[4] = {eye[0], eye[1], eye[2], 1.f}, o[4];
    q[axis] = q[axis] + size * 0.5f;
    mul4(cam->proj, q, o);
    return axis == 0 ? o[0] / o[3] * 0.5f + 0.5f - u : o[1] / o[3] * 0.5f + 0.5f - v;
}

/* mode 0 Gaussian depth, 1 bilateral depth, 2 Gaussian thickness */
static void blur(int mode, int axis, const float *src, const float *dsrc, float *dst, int W, int H, const cam_t *cam,
                 float size, float bscale, float falloff) {
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int64_t id = (int64_t)y * W + x;
            float cur = dsrc[id];
            if (cur == 1.f) {
                dst[id] = mode == 2 ? 0.f : 1.f;
                continue;
            }
            float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H, eye[3];
            uv_to_eye(cam, u, v, cur, eye);
            int texn = axis == 0 ? W : H;
            float ext = screen_extent(cam, eye, size, axis, u, v), acc = 0.f, wsum = 0.f;
            if (mode == 1) {
                int R = (int)(ext * (float)texn);
                R = R > 35 ? 35 : (R < 1 ? 1 : R);
                for (int p = -R; p <= R; p++) {
                    float s = axis == 0 ? tex(src, W, H, x + p, y) : tex(src, W, H, x, y + p);
                    if (s < 1.f) {
                        float rr = (float)p * bscale, w = expf(-rr * rr);
                        float r2 = (s - cur) * falloff, g = expf(-r2 * r2);
                        acc = acc + s * w * g;
                        wsum = wsum + w * g;
                    }
                }
                dst[id] = wsum == 0.f ? 1.f : acc / wsum;
                continue;
            }
            int ks = (int)(ext * (float)texn) * 2 + 1;
            ks = ks > 51 ? 51 : (ks < 3 ? 3 : ks);
            float sd = (float)(ks - 1) / 6.f, sd2 = sd * sd;
            int R = ks / 2;
            for (int p = -R; p <= R; p++) {
                float s = axis == 0 ? tex(src, W, H, x + p, y) : tex(src, W, H, x, y + p);
                if (mode == 2 || s < 1.f) {
                    float w = expf((float)(-p * p) / sd2 * 0.5f);
                    wsum = wsum + w;
                    acc = acc + s * w;
                }
            }
            dst[id] = acc / wsum;
        }
}

/* ---- normals ----------------------------------------------------------- */
static void eye_at(const cam_t *cam, const float *depth, int W, int H, int x, int y, float *e) {
    float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
    uv_to_eye(cam, u, v, tex(depth, W, H, x, y), e);
}

static void normals(const float *depth, float *nd, int W, int H, const cam_t *cam) {
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int64_t id = (int64_t)y * W + x;
            float d = depth[id];
            float *o = nd + 4 * id;
            if (d == 1.f) {
                o[0] = o[1] = o[2] = 0.f;
                o[3] = 1.f;
                continue;
            }
            float p[3], a[3], b[3], ddx[3], ddx2[3], ddy[3], ddy2[3], n[3], w[4];
            eye_at(cam, depth, W, H, x, y, p);
            eye_at(cam, depth, W, H, x + 1, y, a);
            eye_at(cam, depth, W, H, x - 1, y, b);
            for (int k = 0; k < 3; k++) { ddx[k] = a[k] - p[k]; ddx2[k] = p[k] - b[k]; }
            if (fabsf(ddx[2]) > fabsf(ddx2[2])) memcpy(ddx, ddx2, sizeof(ddx));
            eye_at(cam, depth, W, H, x, y + 1, a);
            eye_at(cam, depth, W, H, x, y - 1, b);
            for (int k = 0; k < 3; k++) { ddy[k] = a[k] - p[k]; ddy2[k] = p[k] - b[k]; }
            if (fabsf(ddy2[2]) < fabsf(ddy[2])) memcpy(ddy, ddy2, sizeof(ddy));
            cross3(ddx, ddy, n);
            normalize3(n);
            float n4[4] = {n[0], n[1], n[2], 0.f};
            mul4(cam->view_inv, n4, w);
            o[0] = w[0]; o[1] = w[1]; o[2] = w[2]; o[3] = d;
        }
}

/* ---- shading ------------------------------------------------------------ */
/* Classic Perlin noise as the shader's cnoise computes it: hashes by the
 * permutation polynomial (34x + 10)x mod 289, gradients from the hash folded
 * onto an octahedron, normalised by the Taylor inverse square root, quintic
 * fade, result scaled by 2.2. */
static float mod289(float x) { return x - floorf(x * (1.f / 289.f)) * 289.f; }
static float permute(float x) { return mod289((x * 34.f + 10.f) * x); }
static float fractf(float x) { return x - floorf(x); }
static float fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
static float mixf(float a, float b, float t) { return a * (1.f - t) + b * t; }

static float perlin(float X, float Y, float Z) {
    float i0[3] = {mod289(floorf(X)), mod289(floorf(Y)), mod289(floorf(Z))};
    float i1[3] = {mod289(floorf(X) + 1.f), mod289(floorf(Y) + 1.f), mod289(floorf(Z) + 1.f)};
    float f0[3] = {fractf(X), fractf(Y), fractf(Z)};
    float f1[3] = {f0[0] - 1.f, f0[1] - 1.f, f0[2] - 1.f};
    float n[2][4];
    for (int c = 0; c < 4; c++) {
        int cx = c & 1, cy = c >> 1;
        float hxy = permute(permute(cx ? i1[0] : i0[0]) + (cy ? i1[1] : i0[1]));
        for (int cz = 0; cz < 2; cz++) {
            float h = permute(hxy + (cz ? i1[2] : i0[2]));
            float gx = h * (1.f / 7.f);
            float gy = fractf(floorf(gx) * (1.f / 7.f)) - 0.5f;
            gx = fractf(gx);
            float gz = 0.5f - fabsf(gx) - fabsf(gy);
            float sz = gz <= 0.f ? 1.f : 0.f;
            gx = gx - sz * ((gx < 0.f ? 0.f : 1.f) - 0.5f);
            gy = gy - sz * ((gy < 0.f ? 0.f : 1.f) - 0.5f);
            float norm = 1.79284291400159f - 0.85373472095314f * (gx * gx + gy * gy + gz * gz);
            n[cz][c] = (gx * norm) * (cx ? f1[0] : f0[0]) + (gy * norm) * (cy ? f1[1] : f0[1]) +
                       (gz * norm) * (cz ? f1[2] : f0[2]);
        }
    }
    float fx = fade(f0[0]), fy = fade(f0[1]), fz = fade(f0[2]), nz[4];
    for (int c = 0; c < 4; c++) nz[c] = mixf(n[0][c], n[1][c], fz);
    float ny0 = mixf(nz[0], nz[2], fy), ny1 = mixf(nz[1], nz[3], fy);
    return 2.2f * mixf(ny0, ny1, fx);
}

typedef struct {
    const cam_t *cam;
    int W, H;
    const float *nd;
    const fsim_render_params *p;
} shade_ctx;

static void world_at(const shade_ctx *a, int x, int y, float *w, float *nrm) {
    int cx = clampi(x, 0, a->W - 1), cy = clampi(y, 0, a->H - 1);
    const float *t = a->nd + 4 * ((int64_t)cy * a->W + cx);
    float u = ((float)x + 0.5f) / (float)a->W, v = ((float)y + 0.5f) / (float)a->H, e[3], o[4];
    uv_to_eye(a->cam, u, v, t[3], e);
    float e4[4] = {e[0], e[1], e[2], 1.f};
    mul4(a->cam->view_inv, e4, o);
    w[0] = o[0]; w[1] = o[1]; w[2] = o[2];
    nrm[0] = t[0]; nrm[1] = t[1]; nrm[2] = t[2];
}

static void noisy_pos(const shade_ctx *a, int x, int y, float *out) {
    float w[3], n[3];
    world_at(a, x, y, w, n);
    const fsim_render_params *p = a->p;
    float px = w[0] * p->noise_scale, py = w[1] * p->noise_scale, pz = w[2] * p->noise_scale;
    float noise = perlin(px + p->noise_offset, py, pz) + perlin(-px + p->noise_offset, py + p->noise_offset, pz);
    for (int k = 0; k < 3; k++) out[k] = w[k] + n[k] * noise;
}

static void shade_light(const float *wp, const float *nrm_in, const float *view, const fsim_light *L,
                        const float *mat, const float *spec, float shininess, float *acc) {
    float f2l[3], ld[3], n[3], hw[3];
    for (int k = 0; k < 3; k++) f2l[k] = L->position[k] - wp[k] * L->position[3];
    memcpy(ld, f2l, sizeof(ld));
    normalize3(ld);
    memcpy(n, nrm_in, sizeof(n));
    if (dot3(n, view) < 0.f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
    float lc = dot3(ld, n);
    if (lc < 0.f) return;
    float d2 = sqrtf(dot3(f2l, f2l));
    d2 = d2 * d2;
    for (int k = 0; k < 3; k++) hw[k] = view[k] + ld[k];
    normalize3(hw);
    float shine = dot3(hw, n);
    if (shine < 0.f) shine = 0.f;
    float sp = powf(shine, shininess);
    for (int k = 0; k < 3; k++) acc[k] = acc[k] + L->power_density[k] * (mat[k] * lc + spec[k] * sp) / d2;
}

static void shade(const shade_ctx *a, const float *thick, const float *scene, float *color) {
    const fsim_render_params *p = a->p;
    const float *bg = p->background;
    float diffuse[4] = {p->particle_color[0], p->particle_color[1], p->particle_color[2], 1.f};
    for (int y = 0; y < a->H; y++)
        for (int x = 0; x < a->W; x++) {
            int64_t id = (int64_t)y * a->W + x;
            const float *t = a->nd + 4 * id;
            float *o = color + 4 * id;
            if (t[3] == 1.f || (scene && !(t[3] < scene[id]))) {
                memcpy(o, bg, 4 * sizeof(float));
                continue;
            }
            float wp[3], n[3];
            world_at(a, x, y, wp, n);
            if (p->noise_enabled) {
                float c0[3], q[3], ddx[3], ddx2[3], ddy[3], ddy2[3], nn[3];
                noisy_pos(a, x, y, c0);
                noisy_pos(a, x + 1, y, q);
                for (int k = 0; k < 3; k++) ddx[k] = q[k] - c0[k];
                noisy_pos(a, x - 1, y, q);
                for (int k = 0; k < 3; k++) ddx2[k] = c0[k] - q[k];
                if (fabsf(ddx[2]) > fabsf(ddx2[2])) memcpy(ddx, ddx2, sizeof(ddx));
                noisy_pos(a, x, y + 1, q);
                for (int k = 0; k < 3; k++) ddy[k] = q[k] - c0[k];
                noisy_pos(a, x, y - 1, q);
                for (int k = 0; k < 3; k++) ddy2[k] = c0[k] - q[k];
                if (fabsf(ddy2[2]) < fabsf(ddy[2])) memcpy(ddy, ddy2, sizeof(ddy));
                cross3(ddx, ddy, nn);
                normalize3(nn);
                float s = p->noise_strength;
                for (int k = 0; k < 3; k++) n[k] = n[k] * (1.f - s) + nn[k] * s;
                normalize3(n);
            }
            float c[4] = {0.f, 0.f, 0.f, diffuse[3]};
            if (p->transparency_enabled) c[3] = expf(-p->transparency * thick[id]);
            float view[3] = {a->cam->pos[0] - wp[0], a->cam->pos[1] - wp[1], a->cam->pos[2] - wp[2]};
            normalize3(view);
            for (int l = 0; l < p->num_lights; l++)
                shade_light(wp, n, view, &p->lights[l], diffuse, p->specular_color, p->shininess, c);
            if (p->transparency_enabled) {
                float al = c[3];
                for (int k = 0; k < 4; k++) o[k] = c[k] * (1.f - al) + bg[k] * al;
            } else {
                memcpy(o, c, sizeof(c));
            }
        }
}

/* One frame; every output image is W * H (x4 for nd and color) floats. */
int render_oracle_frame(const fsim_particle_gfx *pt, int64_t n, const fsim_camera *camera,
                        const fsim_render_params *p, const float *scene, int W, int H, float *raw, float *depth,
                        float *thick, float *nd, float *color) {
    if (!camera || !p || W <= 0 || H <= 0 || !raw || !depth || !thick || !nd || !color) return -1;
    cam_t cam = {camera->view, camera->view_inv, camera->proj, camera->proj_inv, camera->position};
    const int64_t np = (int64_t)W * H;
    float *tmp = (float *)malloc((size_t)np * sizeof(float));
    if (!tmp) return -2;
    const float r = p->particle_radius;
    for (int64_t i = 0; i < np; i++) raw[i] = 1.f;
    splat_depth(pt, n, p->spray_enabled ? 1 : 0, p->spray_density_threshold, &cam, r, W, H, raw);
    int mode = p->bilateral_filter ? 1 : 0;
    blur(mode, 0, raw, raw, tmp, W, H, &cam, p->smoothing_size, p->blur_scale, p->blur_depth_falloff);
    blur(mode, 1, tmp, tmp, depth, W, H, &cam, p->smoothing_size, p->blur_scale, p->blur_depth_falloff);
    if (p->spray_enabled) splat_depth(pt, n, 2, p->spray_density_threshold, &cam, r, W, H, depth);
    for (int64_t i = 0; i < np; i++) thick[i] = 0.f;
    if (p->transparency_enabled) {
        splat_thickness(pt, n, &cam, r, W, H, scene, thick);
        blur(2, 0, thick, depth, tmp, W, H, &cam, p->transparency_blur_size, 0.f, 0.f);
        blur(2, 1, tmp, depth, thick, W, H, &cam, p->transparency_blur_size, 0.f, 0.f);
    }
    normals(depth, nd, W, H, &cam);
    shade_ctx a = {&cam, W, H, nd, p};
    shade(&a, thick, scene, color);
    free(tmp);
    return 0;
}
