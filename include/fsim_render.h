/* fsim_render.h -- headless screen-space fluid renderer on the GPU.
 *
 * The reference draws the particles with OpenGL in FluidSurfaceGfx::render
 * (src/Application/gfx/gfx3D/fluidSurfaceGfx.cpp:81-204): a depth splat of
 * spherical sprites (shaders/particle_sprites.vs, particle_sprites_depth.fs),
 * a separable Gaussian or bilateral depth smoothing (gaussian.fs,
 * bilateral.fs), spray particles splatted on top, an additive thickness splat
 * and its blur (particle_sprites_thickness.fs, gaussian_thickness.fs), normal
 * reconstruction from the smoothed depth (normal_depth.fs) and Blinn-Phong
 * shading with surface noise and thickness-based transparency
 * (shadedDepth.fs).  This library runs the same passes as CUDA kernels into
 * device images; there is no window, swapchain or graphics API.  Images are
 * width x height, row 0 at the bottom (OpenGL window convention), row-major.
 *
 * Particles come from fsim_fill_gfx (fsim_particle_gfx: pos, |v|, density).
 * Every call returns 0 or a negative FSIM_E_* code (include/fsim.h).
 */
#ifndef FSIM_RENDER_H
#define FSIM_RENDER_H

#include <stdint.h>

#include "fsim.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Camera3D uniforms (engineUtils/camera3D.hpp:103-125): column-major 4x4
 * matrices as glm stores them (element [col * 4 + row]). */
typedef struct fsim_camera {
    float view[16];        /* glm::lookAt */
    float view_inv[16];
    float proj[16];        /* glm::perspective(fov, aspect, near, far) */
    float proj_inv[16];
    float position[4];     /* camera.position (world, w = 1) */
} fsim_camera;

/* renderer::Light (engineUtils/lights.hpp:16-26): w = 0 directional, 1 point. */
typedef struct fsim_light {
    float position[4];
    float power_density[3];
} fsim_light;

#define FSIM_RENDER_MAX_LIGHTS 8

/* FluidSurfaceGfx parameters (fluidSurfaceGfx.h:26-41) and the material of
 * its shaded quad (fluidSurfaceGfx.cpp:24-26). */
typedef struct fsim_render_params {
    float particle_radius;         /* SimulationConfig::particleRadius */
    float particle_color[3];       /* "Fluid color" (0, 0.4, 0.95) */
    float specular_color[3];       /* (1.2, 1.2, 1.2) */
    float shininess;               /* 80 */
    int bilateral_filter;          /* "Bilateral filter" (0: Gaussian) */
    float smoothing_size;          /* "Gaussian smoothing" 2.4 (world units) */
    float blur_scale;              /* "Blur scale" 0.083 */
    float blur_depth_falloff;      /* "Blur depth falloff" 1100 */
    int spray_enabled;             /* "Spray" 1 */
    float spray_density_threshold; /* "Spray density threashold" 1.2 */
    int transparency_enabled;      /* "Transparent fluid" 1 */
    float transparency_blur_size;  /* "Fluid thickness blur size" 2.4 */
    float transparency;            /* "Fluid transparency" 1.334 */
    int noise_enabled;             /* "Fluid surface noise" 1 */
    float noise_scale;             /* "Noise scale" 0.956 */
    float noise_strength;          /* "Noise strength" 0.123 */
    float noise_offset;            /* advanced by the caller: += speed * 10 * frame time */
    int num_lights;
    fsim_light lights[FSIM_RENDER_MAX_LIGHTS];
    float background[4];           /* the render target under the fluid (RGBA) */
} fsim_render_params;

/* Fills p with the reference GUI's defaults (the values quoted above) and its
 * four point lights (simulationGfx3D.cpp:249-252). */
void fsim_render_default_params(fsim_render_params *p);

/* Builds a camera as Camera3D does: lookAt(eye, eye + dir(yaw, pitch), up) and
 * perspective(fov_deg, aspect, near, far); matrices computed in double and
 * stored as float. */
void fsim_render_camera(fsim_camera *cam, const double eye[3], double yaw_deg, double pitch_deg, double fov_deg,
                        double aspect, double z_near, double z_far);

enum fsim_render_image {
    FSIM_IMG_COLOR = 0,         /* float4 RGBA: the composited frame */
    FSIM_IMG_DEPTH = 1,         /* float: smoothed fluid depth + spray, 1 = empty */
    FSIM_IMG_THICKNESS = 2,     /* float: blurred thickness */
    FSIM_IMG_NORMAL_DEPTH = 3,  /* float4: world normal, depth (normalAndDepthTexture) */
    FSIM_IMG_RAW_DEPTH = 4      /* float: sprite depth before smoothing */
};

typedef struct fsim_renderer fsim_renderer;

int fsim_render_create(int width, int height, fsim_renderer **out);
int fsim_render_destroy(fsim_renderer *r);
const char *fsim_render_last_error(fsim_renderer *r);

/* One frame.  particles: n records on the device (fsim_fill_gfx with
 * FSIM_DEVICE), or on the host with where = FSIM_HOST (copied first).
 * scene_depth: optional device depth image (width x height floats, window
 * depth in [0, 1]) of the other objects of the scene, which the thickness
 * splat and the final composite are depth-tested against; NULL = empty scene.
 * stream: a cudaStream_t or NULL for the renderer's own stream. */
int fsim_render_frame(fsim_renderer *r, const fsim_particle_gfx *particles, int64_t n, int where,
                      const fsim_camera *cam, const fsim_render_params *params, const float *scene_depth,
                      void *stream);

/* Renders the particles of a simulation context (fsim_fill_gfx into the
 * renderer's own device buffer, then fsim_render_frame on the context's stream). */
int fsim_render_ctx(fsim_renderer *r, fsim_ctx *ctx, const fsim_camera *cam, const fsim_render_params *params,
                    const float *scene_depth);

/* Copies an image out (FSIM_HOST or FSIM_DEVICE destination); waits for the frame. */
int fsim_render_read(fsim_renderer *r, int image, void *dst, int where);

/* Time of the last frame's kernels (CUDA events), milliseconds, and the number
 * of kernels it launched. */
int fsim_render_stats(fsim_renderer *r, float *ms, int *launches);

#ifdef __cplusplus
}
#endif

#endif
