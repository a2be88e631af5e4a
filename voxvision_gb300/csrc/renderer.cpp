/*
 * renderer.cpp -- the vox_render context API (src/voxrnd/renderer.h) over the
 * GPU render path of voxtrees_cuda.cu.
 *
 * vox_render (renderer.c:200-319) draws a whole frame: the scene tree is
 * uploaded once per vox_context_set_scene, the camera state is read from the
 * built-in camera object, and one fused kernel draws the ARGB frame into the
 * context's device frame.  A camera of any other class (one
 * whose iface is not the built-in simple or doom camera's) is asked for every
 * pixel's direction through its own screen2world on the host threads, as the
 * reference's tasks ask it, and the frame is drawn from that ray buffer.
 * vox_redraw (renderer.c:321-327) then copies the frame into the page-locked
 * host buffer returned by vox_context_pixels.  Instead of an SDL surface the
 * context owns a headless frame.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../../include/voxrnd.h"
#include "../../include/voxtrees_cuda.h"
#include "frame_memo.h"
#include "lights_internal.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

extern "C" int vox_camera_gpu_state(const struct vox_camera *cam, float *position, float *rotation,
                                    float *mul, float *xsub, float *ysub, float *sinphi, float *cosphi,
                                    float *k);
extern "C" int vox_cuda_render_quality_device(const vox_cuda_tree *tree, const vox_cuda_camera *camera,
                                              uint32_t w, uint32_t h, unsigned int quality,
                                              const uint8_t *texture, uint32_t *argb, void *stream);

struct vox_rnd_ctx {
    unsigned int w = 0, h = 0;
    struct vox_node *scene = nullptr;
    struct vox_camera *camera = nullptr;
    unsigned int quality = VOX_QUALITY_ADAPTIVE;   // renderer.c:78
    vox_cuda_tree *tree = nullptr;
    bool tex_dirty = true;
    uint8_t texture[32768];
    uint8_t *d_tex = nullptr;
    uint32_t *d_frame = nullptr;                   // the frame vox_render draws (device; zeroed at creation)
    uint32_t *pixels = nullptr;                    // what vox_context_pixels returns (page-locked)
    cudaStream_t stream = nullptr;
    int status = VOX_CUDA_OK;
    struct vox_light_manager *lights = nullptr;    // renderer.h:66
    vox_cuda_lights *d_lights = nullptr;           // its device copy
    uint64_t d_lights_version = 0;                 // the manager's version that copy holds
    float *h_rays = nullptr;                       // pixel directions of a host-computed camera (pinned)
    float *d_rays = nullptr;                       // their device copy
    vox::FrameMemo memo{true, 0, 0, 0, 0};         // what d_frame holds (zeroed at creation)
    vox::FrameMemo shown{true, 0, 0, 0, 0};        // what `pixels` holds (zeroed at creation)
};

namespace {

// splitmix64, seed 7: the default texture (the reference's vn3d noise is not
// part of this library).
void default_texture(uint8_t *tex)
{
    uint64_t s = 7;
    for (int i = 0; i < 32768; i++) {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        tex[i] = (uint8_t)(z >> 56);
    }
}

void release(vox_rnd_ctx *c)
{
    if (c->d_lights) vox_cuda_lights_free(c->d_lights);
    if (c->tree) vox_cuda_tree_free(c->tree);
    if (c->d_tex) cudaFree(c->d_tex);
    if (c->d_frame) cudaFree(c->d_frame);
    if (c->pixels) cudaFreeHost(c->pixels);
    if (c->h_rays) cudaFreeHost(c->h_rays);
    if (c->d_rays) cudaFree(c->d_rays);
    if (c->stream) cudaStreamDestroy(c->stream);
}

// Every pixel's direction from the camera's own screen2world, rows dealt to
// the host threads (the reference calls it from its parallel tasks too), then
// copied to the device on the context's stream.
int fill_rays(vox_rnd_ctx *c)
{
    const size_t n = (size_t)c->w * c->h * 3;
    if (!c->h_rays && cudaMallocHost(&c->h_rays, n * sizeof(float)) != cudaSuccess) {
        c->h_rays = nullptr;
        return VOX_CUDA_ENOMEM;
    }
    if (!c->d_rays && cudaMalloc(&c->d_rays, n * sizeof(float)) != cudaSuccess) {
        c->d_rays = nullptr;
        return VOX_CUDA_ENOMEM;
    }
    struct vox_camera *cam = c->camera;
    std::atomic<unsigned int> next{0};
    auto rows = [&]() {
        for (unsigned int y; (y = next.fetch_add(1)) < c->h;)
            for (unsigned int x = 0; x < c->w; x++)
                cam->iface->screen2world(cam, c->h_rays + 3 * ((size_t)y * c->w + x), (int)x, (int)y);
    };
    unsigned int nt = std::min(std::max(1u, std::thread::hardware_concurrency()), std::max(1u, c->h / 16));
    std::vector<std::thread> pool;
    try {
        for (unsigned int i = 1; i < nt; i++) pool.emplace_back(rows);
    } catch (...) {
        // fewer threads: rows are dealt dynamically, the rest draw them all
    }
    rows();
    for (auto &th : pool) th.join();
    if (cudaMemcpyAsync(c->d_rays, c->h_rays, n * sizeof(float), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
        return VOX_CUDA_ECUDA;
    return VOX_CUDA_OK;
}

}  // namespace

EXPORT struct vox_rnd_ctx *vox_make_context_headless(unsigned int width, unsigned int height)
{
    if (width == 0 || height == 0 || (width & 0xF) || (height & 0x3)) return nullptr;  // renderer.c:97-100
    vox_rnd_ctx *c = new (std::nothrow) vox_rnd_ctx();
    if (!c) return nullptr;
    c->w = width;
    c->h = height;
    default_texture(c->texture);
    size_t bytes = (size_t)width * height * 4;
    void *px = nullptr;
    if (cudaMallocHost(&px, bytes) != cudaSuccess) px = nullptr;
    c->pixels = static_cast<uint32_t *>(px);
    if (!c->pixels || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_tex, 32768) != cudaSuccess || cudaMalloc(&c->d_frame, bytes) != cudaSuccess ||
        cudaMemsetAsync(c->d_frame, 0, bytes, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        release(c);
        delete c;
        return nullptr;
    }
    std::memset(c->pixels, 0, bytes);
    return c;
}

EXPORT void vox_destroy_context(struct vox_rnd_ctx *ctx)
{
    if (!ctx) return;
    release(ctx);
    delete ctx;
}

EXPORT void vox_context_set_scene(struct vox_rnd_ctx *ctx, struct vox_node *scene)
{
    ctx->scene = scene;
    if (ctx->tree) {
        vox_cuda_tree_free(ctx->tree);
        ctx->tree = nullptr;
    }
}

EXPORT void vox_context_set_camera(struct vox_rnd_ctx *ctx, struct vox_camera *camera)
{
    ctx->camera = camera;
    camera->iface->set_window_size(camera, (int)ctx->w, (int)ctx->h);   // renderer.c:163-167
}

/* renderer.c:179-195 */
EXPORT int vox_context_set_quality(struct vox_rnd_ctx *ctx, unsigned int quality)
{
    if ((quality & VOX_QUALITY_RM_MASK) && ((quality & VOX_QUALITY_MODE_MASK) != VOX_QUALITY_ADAPTIVE))
        return 0;
    if ((quality & VOX_QUALITY_MODE_MASK) > VOX_QUALITY_ADAPTIVE) return 0;
    if ((quality & VOX_QUALITY_RM_MASK) > VOX_QUALITY_RAY_MERGE_ACCURATE) return 0;
    ctx->quality = quality;
    return 1;
}

EXPORT void vox_context_set_texture(struct vox_rnd_ctx *ctx, const uint8_t *texture)
{
    std::memcpy(ctx->texture, texture, 32768);
    ctx->tex_dirty = true;
}

EXPORT void vox_context_set_light_manager(struct vox_rnd_ctx *ctx, struct vox_light_manager *light_manager)
{
    ctx->lights = light_manager;   // renderer.c:174-177; copied to the device at the next vox_render
}

EXPORT void vox_render(struct vox_rnd_ctx *ctx)
{
    ctx->status = VOX_CUDA_EINVAL;
    if (!ctx->camera) return;
    vox_cuda_camera cam;
    std::memset(&cam, 0, sizeof cam);
    int kind = vox_camera_gpu_state(ctx->camera, cam.position, cam.rotation, &cam.mul, &cam.xsub, &cam.ysub,
                                    &cam.sinphi, &cam.cosphi, &cam.k);
    cam.kind = kind;        // < 0: a class the device cannot compute
    if (!ctx->tree) {
        int rc = vox_cuda_tree_upload(ctx->scene, &ctx->tree);
        if (rc) { ctx->status = rc; return; }
    }
    if (ctx->tex_dirty) {
        if (cudaMemcpyAsync(ctx->d_tex, ctx->texture, 32768, cudaMemcpyHostToDevice, ctx->stream) !=
            cudaSuccess) { ctx->status = VOX_CUDA_ECUDA; return; }
        ctx->tex_dirty = false;
    }
    if (ctx->lights && (!ctx->d_lights || ctx->d_lights_version != ctx->lights->version)) {
        // the manager changed since the last frame (or is new): upload it again
        if (ctx->d_lights) {
            cudaStreamSynchronize(ctx->stream);
            vox_cuda_lights_free(ctx->d_lights);
            ctx->d_lights = nullptr;
        }
        int rc = vox_cuda_lights_upload(ctx->lights, &ctx->d_lights);
        if (rc) { ctx->status = rc; return; }
        ctx->d_lights_version = ctx->lights->version;
    }
    uint32_t *target = ctx->d_frame;
    const vox_cuda_lights *lights = ctx->lights ? ctx->d_lights : nullptr;
    int rc;
    if (kind < 0) {
        // the previous frame's directions may still be in use: wait for it first
        if (ctx->h_rays && cudaStreamSynchronize(ctx->stream) != cudaSuccess) { ctx->status = VOX_CUDA_ECUDA; return; }
        rc = fill_rays(ctx);
        if (rc) { ctx->status = rc; return; }
        vox_dot origin;
        ctx->camera->iface->get_position(ctx->camera, origin);   // renderer.c:231
        vox_cuda_camera at;
        std::memset(&at, 0, sizeof at);
        at.kind = VOX_CUDA_CAMERA_SIMPLE;   // only its position is read
        for (int a = 0; a < 3; a++) at.position[a] = origin[a];
        rc = render_frame_memo(ctx->tree, &at, ctx->d_rays, ctx->w, ctx->h, ctx->quality, ctx->d_tex, lights,
                               target, ctx->stream, &ctx->memo);
    } else {
        // the frame is the context's own: the next one clears only what this
        // one drew outside the new tree rectangle
        rc = render_frame_memo(ctx->tree, &cam, nullptr, ctx->w, ctx->h, ctx->quality, ctx->d_tex, lights, target,
                               ctx->stream, &ctx->memo);
    }
    if (rc) { ctx->status = rc; return; }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        ctx->status = VOX_CUDA_ECUDA;
        return;
    }
    ctx->status = VOX_CUDA_OK;
}

// The last frame into the buffer vox_context_pixels returns, by the copy
// engine.  Both frames are zero outside their tree rectangles when their
// memos are valid, so only the box covering both rectangles is copied.
EXPORT void vox_redraw(struct vox_rnd_ctx *ctx)
{
    const size_t w = ctx->w, row = w * 4;
    const vox::FrameMemo &now = ctx->memo, &was = ctx->shown;
    cudaError_t e = cudaSuccess;
    if (!now.valid || !was.valid) {
        e = cudaMemcpyAsync(ctx->pixels, ctx->d_frame, row * ctx->h, cudaMemcpyDeviceToHost, ctx->stream);
    } else {
        uint32_t x0 = ctx->w, y0 = ctx->h, x1 = 0, y1 = 0;
        for (const vox::FrameMemo *m : {&now, &was})
            if (m->x1 > m->x0 && m->y1 > m->y0) {
                x0 = std::min(x0, m->x0); y0 = std::min(y0, m->y0);
                x1 = std::max(x1, m->x1); y1 = std::max(y1, m->y1);
            }
        if (x1 > x0) {
            size_t off = (size_t)y0 * w + x0;
            e = cudaMemcpy2DAsync(ctx->pixels + off, row, ctx->d_frame + off, row, (size_t)(x1 - x0) * 4, y1 - y0,
                                  cudaMemcpyDeviceToHost, ctx->stream);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        ctx->status = VOX_CUDA_ECUDA;
        ctx->shown = vox::FrameMemo{false, 0, 0, 0, 0};   // unknown: the next redraw copies all
        return;
    }
    ctx->shown = now;
}

EXPORT const uint32_t *vox_context_pixels(const struct vox_rnd_ctx *ctx) { return ctx->pixels; }

EXPORT int vox_context_status(const struct vox_rnd_ctx *ctx) { return ctx->status; }

/* ---- collision detector (src/voxrnd/cd.c) ---- */

struct vox_cd {                 /* cd.c:6-11 */
    struct vox_camera *camera;
    struct vox_rnd_ctx *ctx;
    vox_dot last_position;
    float camera_radius;
};

EXPORT struct vox_cd *vox_make_cd(void)
{
    struct vox_cd *cd = static_cast<struct vox_cd *>(std::calloc(1, sizeof(struct vox_cd)));
    return cd;
}

EXPORT void vox_cd_attach_camera(struct vox_cd *cd, struct vox_camera *camera, float radius)
{
    cd->camera = camera;
    cd->camera_radius = radius;
    camera->iface->get_position(camera, cd->last_position);
}

EXPORT void vox_cd_attach_context(struct vox_cd *cd, struct vox_rnd_ctx *ctx) { cd->ctx = ctx; }

/* cd.c:29-32: a stub in the reference as well. */
EXPORT void vox_cd_gravity(struct vox_cd *cd, const vox_dot gravity) {}

/* cd.c:34-55: if the camera moved into the scene (a ball of the camera's
 * radius meets a voxel), put it back where it was; otherwise remember the
 * new position.  The ball query runs on the GPU against the context's tree. */
EXPORT void vox_cd_collide(struct vox_cd *cd)
{
    struct vox_camera *camera = cd->camera;
    struct vox_rnd_ctx *ctx = cd->ctx;
    if (!camera || !ctx) return;
    vox_dot position;
    camera->iface->get_position(camera, position);
    if (std::memcmp(position, cd->last_position, sizeof(vox_dot)) == 0) return;
    if (!ctx->tree && vox_cuda_tree_upload(ctx->scene, &ctx->tree) != VOX_CUDA_OK) return;
    uint8_t hit = 0;
    if (vox_cuda_ball_batch(ctx->tree, position, &cd->camera_radius, 1, &hit, ctx->stream) != VOX_CUDA_OK) return;
    if (hit)
        camera->iface->set_property_dot(camera, "position", cd->last_position);
    else
        std::memcpy(cd->last_position, position, sizeof(vox_dot));
}
