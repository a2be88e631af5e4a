/*
 * cameras.c -- the reference's two camera classes, built in.
 *
 * Object layouts, method order and float arithmetic follow
 * src/voxrnd/simple-camera.c, src/voxrnd/doom-camera.c, src/voxrnd/camera.c
 * and the scalar src/voxrnd/vect-ops.c, so a camera set up through these
 * methods holds the same state as the reference's, and the GPU's
 * screen2world (traverse.cuh) reproduces the host method bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/voxrnd.h"

#define EXPORT __attribute__((visibility("default")))

/* simple-camera.c:10-17 */
struct simple_camera {
    struct vox_camera_interface *iface;
    float xsub, ysub;
    vox_dot position;
    vox_quat rotation;
    float mul, fov;
};

/* doom-camera.c:8-15 */
struct doom_camera {
    struct vox_camera_interface *iface;
    float xsub, ysub;
    vox_dot position;
    float phi, sinphi, cosphi, k;
    float mul, fov;
};

/* ------------------------------------------------------------ vector math */

/* v1 x v2 (vect-ops.c:7-15) */
static void cross3(const float *a, const float *b, float *r)
{
    float ax = a[0], ay = a[1], az = a[2];
    float bx = b[0], by = b[1], bz = b[2];
    r[0] = ay * bz - az * by;
    r[1] = -ax * bz + az * bx;
    r[2] = ax * by - ay * bx;
}

/* q1 * q2 (vect-ops.c:17-26); res may alias either operand. */
static void quat_mul(const float *q1, const float *q2, float *res)
{
    float w1 = q1[0], x1 = q1[1], y1 = q1[2], z1 = q1[3];
    float w2 = q2[0], x2 = q2[1], y2 = q2[2], z2 = q2[3];
    res[0] = w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2;
    res[1] = y1 * z2 - z1 * y2 + x1 * w2 + w1 * x2;
    res[2] = z1 * x2 - x1 * z2 + y1 * w2 + w1 * y2;
    res[3] = x1 * y2 - y1 * x2 + z1 * w2 + w1 * z2;
}

/* v + w t + q x t with t = 2 (q x v)  (vect-ops.c:28-36) */
static void rotate3(const float *q, const float *v, float *res)
{
    float t[3], u[3];
    cross3(q + 1, v, t);
    for (int i = 0; i < 3; i++) t[i] = t[i] * 2.0f;
    cross3(q + 1, t, u);
    for (int i = 0; i < 3; i++) res[i] = v[i] + q[0] * t[i] + u[i];
}

static void normalize4(float *q)
{
    float s = 0;
    for (int i = 0; i < 4; i++) s += q[i] * q[i];
    float n = sqrtf(s);
    for (int i = 0; i < 4; i++) q[i] /= n;
}

static void set_identity(float *q)
{
    q[0] = 1; q[1] = 0; q[2] = 0; q[3] = 0;
}

/* The vector helpers libvoxrnd exports for camera modules (vect-ops.h:13-64,
 * vect-ops.c:17-70), so that a camera class built against the reference
 * links against this library too.  The same arithmetic as the built-in
 * cameras use. */
EXPORT void vox_quat_mul(const vox_quat q1, const vox_quat q2, vox_quat res) { quat_mul(q1, q2, res); }

EXPORT void vox_rotate_vector(const vox_quat base, const vox_dot vector, vox_dot res)
{
    rotate3(base, vector, res);
}

/* The vector part of `vector` rotated into res[1..3]; res[0] is left as it is. */
EXPORT void vox_rotate_vector_q(const vox_quat base, const vox_quat vector, vox_quat res)
{
    rotate3(base, vector + 1, res + 1);
}

EXPORT void vox_quat_normalize(vox_quat quat) { normalize4(quat); }

EXPORT void vox_dot_normalize(vox_dot dot)
{
    float s = 0;
    for (int i = 0; i < 3; i++) s += dot[i] * dot[i];
    float n = sqrtf(s);
    for (int i = 0; i < 3; i++) dot[i] /= n;
}

EXPORT void vox_quat_set_identity(vox_quat quat) { set_identity(quat); }

/* set_window_size of both classes (simple-camera.c:120-136) */
static void window_params(float fov, int w, int h, float *xsub, float *ysub, float *mul)
{
    if (w > h) {
        *xsub = fov;
        *ysub = fov * h / w;
        *mul = fov * 2 / w;
    } else {
        *ysub = fov;
        *xsub = fov * w / h;
        *mul = fov * 2 / h;
    }
}

static void dummy_void(void) {}

static void dummy_dot(const struct vox_camera *c, vox_dot d)
{
    (void)c;
    memset(d, 0, sizeof(vox_dot));
}

/* ------------------------------------------------------------ simple */

static void simple_screen2world(const struct vox_camera *cam, vox_dot ray, int sx, int sy)
{
    const struct simple_camera *c = (const void *)cam;
    vox_dot v = {c->mul * sx - c->xsub, 1, c->ysub - c->mul * sy};
    rotate3(c->rotation, v, ray);
}

static void simple_get_position(const struct vox_camera *cam, vox_dot res)
{
    const struct simple_camera *c = (const void *)cam;
    memcpy(res, c->position, sizeof(vox_dot));
}

static void simple_move_camera(struct vox_camera *cam, const vox_dot delta)
{
    struct simple_camera *c = (void *)cam;
    vox_dot d;
    rotate3(c->rotation, delta, d);
    for (int i = 0; i < 3; i++) c->position[i] = c->position[i] + d[i];
}

/* Rotate about the camera's own z, then y, then x axis (simple-camera.c:48-104). */
static void simple_rotate_camera(struct vox_camera *cam, const vox_dot delta)
{
    struct simple_camera *c = (void *)cam;
    static const float axes[3][4] = {{0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    for (int i = 2; i >= 0; i--) {
        float r[4];
        r[0] = 0;
        rotate3(c->rotation, axes[i] + 1, r + 1);   /* the axis in world space */
        float s = sinf(delta[i] / 2), co = cosf(delta[i] / 2);
        for (int j = 1; j < 4; j++) r[j] = s * r[j];
        r[0] = co;
        quat_mul(r, c->rotation, c->rotation);
    }
    normalize4(c->rotation);
}

static void simple_look_at(struct vox_camera *cam, const vox_dot coord)
{
    struct simple_camera *c = (void *)cam;
    vox_dot sub, rot;
    for (int i = 0; i < 3; i++) sub[i] = coord[i] - c->position[i];
    set_identity(c->rotation);
    rot[0] = atan2f(sub[2], hypotf(sub[0], sub[1]));
    rot[1] = 0;
    rot[2] = -atan2f(sub[0], sub[1]);
    cam->iface->rotate_camera(cam, rot);
}

static void simple_set_window_size(struct vox_camera *cam, int w, int h)
{
    struct simple_camera *c = (void *)cam;
    window_params(c->fov, w, h, &c->xsub, &c->ysub, &c->mul);
}

static void simple_set_number(struct vox_camera *cam, const char *name, float value)
{
    struct simple_camera *c = (void *)cam;
    if (strcmp(name, "fov") == 0) c->fov = value;
}

static void simple_set_dot(struct vox_camera *cam, const char *name, const vox_dot value)
{
    struct simple_camera *c = (void *)cam;
    if (strcmp(name, "position") == 0) {
        memcpy(c->position, value, sizeof(vox_dot));
    } else if (strcmp(name, "rotation") == 0) {
        float rx[4] = {cosf(value[0] / 2), sinf(value[0] / 2), 0, 0};
        float ry[4] = {cosf(value[1] / 2), 0, sinf(value[1] / 2), 0};
        float rz[4] = {cosf(value[2] / 2), 0, 0, sinf(value[2] / 2)};
        quat_mul(ry, rx, c->rotation);
        quat_mul(rz, c->rotation, c->rotation);
    }
}

static struct vox_camera *simple_construct(const struct vox_camera *old);

static void generic_destroy(struct vox_camera *cam)
{
    free(cam->iface);
    free(cam);
}

static struct vox_camera_interface simple_methods = {
    .set_property_number = simple_set_number,
    .set_property_dot = simple_set_dot,
    .screen2world = simple_screen2world,
    .rotate_camera = simple_rotate_camera,
    .move_camera = simple_move_camera,
    .look_at = simple_look_at,
    .get_position = simple_get_position,
    .set_window_size = simple_set_window_size,
    .construct_camera = simple_construct,
    .destroy_camera = generic_destroy,
};

/* ------------------------------------------------------------ doom */

static void doom_transform(const struct doom_camera *c, const float *v, float *r)
{
    float x = v[0] * c->cosphi - v[1] * c->sinphi;
    float y = v[1] * c->cosphi + v[0] * c->sinphi;
    r[0] = x; r[1] = y; r[2] = v[2];
}

static void doom_screen2world(const struct vox_camera *cam, vox_dot ray, int sx, int sy)
{
    const struct doom_camera *c = (const void *)cam;
    vox_dot d = {c->mul * sx - c->xsub, 1, c->ysub - c->mul * sy};
    d[2] += c->k;
    doom_transform(c, d, ray);
}

static void doom_get_position(const struct vox_camera *cam, vox_dot res)
{
    const struct doom_camera *c = (const void *)cam;
    memcpy(res, c->position, sizeof(vox_dot));
}

static void doom_move_camera(struct vox_camera *cam, const vox_dot delta)
{
    struct doom_camera *c = (void *)cam;
    vox_dot d;
    doom_transform(c, delta, d);
    for (int i = 0; i < 3; i++) c->position[i] = c->position[i] + d[i];
}

static void doom_rotate_camera(struct vox_camera *cam, const vox_dot delta)
{
    struct doom_camera *c = (void *)cam;
    c->k += delta[0];
    c->phi += delta[2];
    c->sinphi = sinf(c->phi);
    c->cosphi = cosf(c->phi);
}

static void doom_look_at(struct vox_camera *cam, const vox_dot coord)
{
    struct doom_camera *c = (void *)cam;
    vox_dot sub;
    for (int i = 0; i < 3; i++) sub[i] = coord[i] - c->position[i];
    c->k = sub[2] / hypotf(sub[0], sub[1]);
    c->phi = -atan2f(sub[0], sub[1]);
    c->cosphi = cosf(c->phi);
    c->sinphi = sinf(c->phi);
}

static void doom_set_window_size(struct vox_camera *cam, int w, int h)
{
    struct doom_camera *c = (void *)cam;
    window_params(c->fov, w, h, &c->xsub, &c->ysub, &c->mul);
}

static void doom_set_number(struct vox_camera *cam, const char *name, float value)
{
    struct doom_camera *c = (void *)cam;
    if (strcmp(name, "fov") == 0) c->fov = value;
}

static void doom_set_dot(struct vox_camera *cam, const char *name, const vox_dot value)
{
    struct doom_camera *c = (void *)cam;
    if (strcmp(name, "position") == 0) {
        memcpy(c->position, value, sizeof(vox_dot));
    } else if (strcmp(name, "rotation") == 0) {
        c->k = value[0];
        c->phi = value[2];
        c->sinphi = sinf(c->phi);
        c->cosphi = cosf(c->phi);
    }
}

static struct vox_camera *doom_construct(const struct vox_camera *old);

static struct vox_camera_interface doom_methods = {
    .set_property_number = doom_set_number,
    .set_property_dot = doom_set_dot,
    .screen2world = doom_screen2world,
    .rotate_camera = doom_rotate_camera,
    .move_camera = doom_move_camera,
    .look_at = doom_look_at,
    .get_position = doom_get_position,
    .set_window_size = doom_set_window_size,
    .construct_camera = doom_construct,
    .destroy_camera = generic_destroy,
};

/* ------------------------------------------------------------ classes */

static struct vox_camera_interface dummy_methods = {
    .set_property_number = (void *)dummy_void,
    .set_property_dot = (void *)dummy_void,
    .screen2world = (void *)dummy_dot,
    .rotate_camera = (void *)dummy_void,
    .move_camera = (void *)dummy_void,
    .look_at = (void *)dummy_void,
    .get_position = dummy_dot,
    .set_window_size = (void *)dummy_void,
    .construct_camera = NULL,
    .destroy_camera = generic_destroy,
};

/* camera.c:6-17: copy the non-NULL methods of iface into the object's table */
EXPORT void vox_use_camera_methods(struct vox_camera *camera, const struct vox_camera_interface *iface)
{
    void *const *src = (void *const *)iface;
    void **dst = (void **)camera->iface;
    for (size_t i = 0; i < sizeof(struct vox_camera_interface) / sizeof(void *); i++)
        if (src[i]) dst[i] = src[i];
}

/* camera.c:37-41 */
EXPORT void vox_init_camera(struct vox_camera *camera)
{
    camera->iface = malloc(sizeof(struct vox_camera_interface));
    memcpy(camera->iface, &dummy_methods, sizeof(struct vox_camera_interface));
}

static struct vox_camera *simple_construct(const struct vox_camera *old)
{
    struct simple_camera *c = malloc(sizeof(*c));
    if (!c) return NULL;
    if (old) {
        memcpy(c, old, sizeof(*c));
    } else {
        memset(c, 0, sizeof(*c));
        c->fov = 1.0f;
        set_identity(c->rotation);
    }
    vox_init_camera((struct vox_camera *)c);
    vox_use_camera_methods((struct vox_camera *)c, &simple_methods);
    return (struct vox_camera *)c;
}

static struct vox_camera *doom_construct(const struct vox_camera *old)
{
    struct doom_camera *c = malloc(sizeof(*c));
    if (!c) return NULL;
    if (old) {
        memcpy(c, old, sizeof(*c));
    } else {
        memset(c, 0, sizeof(*c));
        c->fov = 1.0f;
        c->cosphi = 1.0f;
    }
    vox_init_camera((struct vox_camera *)c);
    vox_use_camera_methods((struct vox_camera *)c, &doom_methods);
    return (struct vox_camera *)c;
}

/* camera.c:43-48: the methods of a camera class by name -- the two built-in
 * classes, or a camera module of that name (modules.c). */
EXPORT struct vox_camera_interface *vox_camera_methods(const char *name)
{
    if (!name) return NULL;
    if (strcmp(name, "simple-camera") == 0) return &simple_methods;
    if (strcmp(name, "doom-camera") == 0) return &doom_methods;
    return (struct vox_camera_interface *)vox_load_module(name, CAMERA_MODULE);
}

/* For the renderer: the vox_cuda_camera state of a built-in camera, or -1
 * for a camera of another class. */
int vox_camera_gpu_state(const struct vox_camera *cam, float *position, float *rotation, float *mul,
                         float *xsub, float *ysub, float *sinphi, float *cosphi, float *k)
{
    if (cam->iface->screen2world == simple_screen2world) {
        const struct simple_camera *c = (const void *)cam;
        memcpy(position, c->position, 12);
        memcpy(rotation, c->rotation, 16);
        *mul = c->mul; *xsub = c->xsub; *ysub = c->ysub;
        *sinphi = 0; *cosphi = 1; *k = 0;
        return 0;
    }
    if (cam->iface->screen2world == doom_screen2world) {
        const struct doom_camera *c = (const void *)cam;
        memcpy(position, c->position, 12);
        rotation[0] = 1; rotation[1] = rotation[2] = rotation[3] = 0;
        *mul = c->mul; *xsub = c->xsub; *ysub = c->ysub;
        *sinphi = c->sinphi; *cosphi = c->cosphi; *k = c->k;
        return 1;
    }
    return -1;
}
