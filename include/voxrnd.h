/*
 * voxrnd.h -- the renderer and camera part of the reference API, as
 * libvoxtrees_cuda exports it (drop-in for src/voxrnd/camera.h and
 * src/voxrnd/renderer.h of shamazmazum/voxvision).
 *
 * Cameras are the reference's two classes, "simple-camera" and
 * "doom-camera", with the same object layout, vtable order and arithmetic
 * (simple-camera.c, doom-camera.c, vect-ops.c); they are built into the
 * library instead of being loaded as plugins.  The renderer keeps the
 * reference's context calls but draws into a headless ARGB8888 frame on the
 * GPU: there is no SDL window or surface (no graphics stack is involved).
 */
#ifndef VOXRND_GB300_H
#define VOXRND_GB300_H

#include <stdint.h>

#include "voxtrees.h"

#ifdef __cplusplus
extern "C" {
#endif

struct vox_camera;

/* camera.h:17-117 (VOX_OBJECT's two property setters come first, object.h). */
struct vox_camera_interface {
    void (*set_property_number)(struct vox_camera *obj, const char *name, float value);
    void (*set_property_dot)(struct vox_camera *obj, const char *name, const vox_dot value);
    void (*screen2world)(const struct vox_camera *camera, vox_dot ray, int sx, int sy);
    void (*rotate_camera)(struct vox_camera *camera, const vox_dot delta);
    void (*move_camera)(struct vox_camera *camera, const vox_dot delta);
    void (*look_at)(struct vox_camera *camera, const vox_dot coord);
    void (*get_position)(const struct vox_camera *camera, vox_dot res);
    void (*set_window_size)(struct vox_camera *camera, int w, int h);
    struct vox_camera *(*construct_camera)(const struct vox_camera *camera);
    void (*destroy_camera)(struct vox_camera *camera);
};

/* camera.h:133-136 */
struct vox_camera {
    struct vox_camera_interface *iface;
};

/* modules.h:15-54: a module is `<name>.so` whose module_init() returns its
 * class and methods; it is looked for in $VOXVISION_MODULES (and in the
 * module directory the library was built with, VOX_MODULE_PATH, if any).
 * NULL when it is not found, cannot be opened or is of another class. */
#define CAMERA_MODULE 0
struct vox_module_methods;
struct vox_module {
    int type;
    struct vox_module_methods *methods;
};
struct vox_module_methods *vox_load_module(const char *name, int type);

/* camera.h:175: methods of a camera class by name: the built-in
 * "simple-camera" and "doom-camera" (which the GPU computes itself), or the
 * camera module of that name (which vox_render asks for every ray). */
struct vox_camera_interface *vox_camera_methods(const char *name);
/* camera.h:146 */
void vox_use_camera_methods(struct vox_camera *camera, const struct vox_camera_interface *iface);
/* camera.h:160 */
void vox_init_camera(struct vox_camera *camera);

/* vect-ops.h:13-64: the vector helpers libvoxrnd exports for camera modules
 * (declared there under VOXRND_SOURCE), so that a camera class built against
 * the reference links against this library.  vox_rotate_vector_q rotates the
 * vector part of `vector` into res[1..3] and leaves res[0] alone. */
void vox_quat_mul(const vox_quat q1, const vox_quat q2, vox_quat res);
void vox_rotate_vector(const vox_quat base, const vox_dot vector, vox_dot res);
void vox_rotate_vector_q(const vox_quat base, const vox_quat vector, vox_quat res);
void vox_quat_normalize(vox_quat quat);
void vox_dot_normalize(vox_dot dot);
void vox_quat_set_identity(vox_quat quat);

/* renderer.h quality flags */
#define VOX_QUALITY_BEST 0x0
#define VOX_QUALITY_FAST 0x1
#define VOX_QUALITY_ADAPTIVE 0x2
#define VOX_QUALITY_RAY_MERGE 0x4
#define VOX_QUALITY_RAY_MERGE_ACCURATE 0x8
#define VOX_QUALITY_RM_MASK 0xC
#define VOX_QUALITY_MODE_MASK 0x3

struct vox_rnd_ctx;

/* Replaces vox_make_context_from_surface / vox_make_context_and_window
 * (renderer.h:145,161): a context drawing into a w x h ARGB8888 frame held
 * by the context (w a multiple of 16, h of 4, else NULL, renderer.c:97-100).
 * The colour texture starts as the 32^3 splitmix64(seed 7) texture; see
 * vox_context_set_texture. */
struct vox_rnd_ctx *vox_make_context_headless(unsigned int width, unsigned int height);
/* renderer.h:201 */
void vox_destroy_context(struct vox_rnd_ctx *ctx);
/* renderer.h:174 */
void vox_context_set_scene(struct vox_rnd_ctx *ctx, struct vox_node *scene);
/* renderer.h:179 (also calls the camera's set_window_size) */
void vox_context_set_camera(struct vox_rnd_ctx *ctx, struct vox_camera *camera);
/* renderer.h:196: 1 if accepted, 0 for an invalid combination */
int vox_context_set_quality(struct vox_rnd_ctx *ctx, unsigned int quality);
/* The 32^3 u8 colour texture (index x*1024 + y*32 + z); the reference
 * generates it with vn3d (renderer.c:54-71), which is not part of this
 * library. */
void vox_context_set_texture(struct vox_rnd_ctx *ctx, const uint8_t *texture);
/* renderer.h:208: render one frame on the GPU into the context's frame. */
void vox_render(struct vox_rnd_ctx *ctx);
/* renderer.h:169: makes the frame of the last vox_render visible through
 * vox_context_pixels. */
void vox_redraw(struct vox_rnd_ctx *ctx);
/* The ARGB8888 frame, pixel (x, y) at [y * width + x]; misses are 0. */
const uint32_t *vox_context_pixels(const struct vox_rnd_ctx *ctx);
/* VOX_CUDA_OK or the error of the last vox_render / vox_redraw. */
int vox_context_status(const struct vox_rnd_ctx *ctx);

/* Light manager (src/voxrnd/lights.h:14-83): an ambient light and soft
 * shadowless lights bound by spheres (brightest at the centre, fading
 * linearly to zero at the surface), kept in an M-tree.  Colours are rgb in
 * [0, 1].  A context with a light manager colours each hit as the reference's
 * get_color does (renderer.c:40-49): min(light, 1) * texel per channel. */
struct vox_light_manager;
/* lights.h:79: ambient light 1, 1, 1; no lights. */
struct vox_light_manager *vox_make_light_manager(void);
/* lights.h:82 */
void vox_destroy_light_manager(struct vox_light_manager *light_manager);
/* lights.h:73: 1 if the colour is valid, 0 otherwise (nothing changes). */
int vox_set_ambient_light(struct vox_light_manager *light_manager, const vox_dot color);
/* lights.h:38: 1 if inserted (valid colour, radius > 0, no light with this
 * centre and radius yet), 0 otherwise. */
int vox_insert_shadowless_light(struct vox_light_manager *light_manager, const vox_dot center, float radius,
                                const vox_dot color);
/* lights.h:48: 1 if a light with this centre and radius was removed. */
int vox_delete_shadowless_light(struct vox_light_manager *light_manager, const vox_dot center, float radius);
/* lights.h:53 */
void vox_delete_shadowless_lights(struct vox_light_manager *light_manager);
/* lights.h:58 */
int vox_shadowless_lights_number(const struct vox_light_manager *light_manager);
/* renderer.h:184: NULL draws without lights (grey texels).  The device copy
 * of the lights follows changes to the manager at the next vox_render. */
void vox_context_set_light_manager(struct vox_rnd_ctx *ctx, struct vox_light_manager *light_manager);

/* Collision detector (src/voxrnd/cd.h:25-60): keeps an attached camera out
 * of the context's scene.  Allocated with malloc; release with free(). */
struct vox_cd;
/* cd.h:25 */
struct vox_cd *vox_make_cd(void);
/* cd.h:32: camera treated as a ball of `radius` */
void vox_cd_attach_camera(struct vox_cd *cd, struct vox_camera *camera, float radius);
/* cd.h:39 */
void vox_cd_attach_context(struct vox_cd *cd, struct vox_rnd_ctx *ctx);
/* cd.h:47: undo the camera's last move if it entered the scene (GPU ball query) */
void vox_cd_collide(struct vox_cd *cd);
/* cd.h:60: no effect, as in the reference */
void vox_cd_gravity(struct vox_cd *cd, const vox_dot gravity);

#ifdef __cplusplus
}
#endif
#endif
