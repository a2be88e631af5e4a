/*
 * voxtrees_cuda.h -- C ABI of libvoxtrees_cuda, the GB300 (sm_103a) ray and
 * ball search over voxtrees octrees.
 *
 * A host tree (struct vox_node, as built by vox_make_tree) is flattened once
 * into one device pool (vox_cuda_tree_upload); batched entry points then run
 * the reference's searches on the GPU:
 *
 *   vox_cuda_ray_batch*   <- vox_ray_tree_intersection  (src/voxtrees/search.h:24-26)
 *   vox_cuda_ball_batch*  <- vox_tree_ball_collidep     (src/voxtrees/search.h:36-37)
 *   vox_cuda_render*      <- vox_render, BEST quality   (src/voxrnd/renderer.h:208,
 *                                                        renderer.c:200-319)
 *
 * Results are bit-identical to the reference's CPU code: the same leaf, the
 * same winning voxel, the same float bits of the intersection point.
 *
 * Conventions.  Every function returns VOX_CUDA_OK (0) or a negative
 * VOX_CUDA_E* code and never aborts.  `stream` is a cudaStream_t passed as
 * void* (NULL = the legacy default stream).  Functions named *_device take
 * device pointers and only enqueue work on `stream`; the others take host
 * pointers, copy inside the call and return when the results are in host
 * memory.  The caller owns host buffers; the library owns the device pool of
 * each uploaded tree.  A tree handle may be used from several threads and
 * streams at once (it is read-only after upload).
 *
 * Leaf identity.  A leaf is reported as its pre-order index among the
 * non-NULL nodes of the uploaded tree (node first, then children 0..7);
 * vox_cuda_tree_node maps it back to the host struct vox_node pointer that
 * vox_ray_tree_intersection would have returned.  VOX_CUDA_MISS marks a miss.
 */
#ifndef VOXTREES_CUDA_H
#define VOXTREES_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VOX_CUDA_OK          0
#define VOX_CUDA_EINVAL     -1   /* bad argument                                   */
#define VOX_CUDA_ENOMEM     -2   /* host or device allocation failed               */
#define VOX_CUDA_ECUDA      -3   /* a CUDA runtime call failed                     */
#define VOX_CUDA_EDEPTH     -4   /* tree deeper than the traversal stack supports  */
#define VOX_CUDA_ESTACK     -5   /* a kernel reported a traversal-stack overflow   */
#define VOX_CUDA_ETOOBIG    -6   /* flattened tree exceeds the 4 GiB pool limit    */
#define VOX_CUDA_EGEOMETRY  -7   /* frame size not a multiple of 16 x 4            */
#define VOX_CUDA_EBUDGET    -8   /* admission budget exceeded                      */
#define VOX_CUDA_ETIMEOUT   -9   /* a bounded wait gave up                         */
#define VOX_CUDA_ENODEV    -10   /* no usable CUDA device                          */
#define VOX_CUDA_ECAPACITY -11   /* request larger than a fixed-capacity entry point */
#define VOX_CUDA_ERANGE    -12   /* checked build: a search met an index outside the tree */

#define VOX_CUDA_MISS       0xFFFFFFFFu
#define VOX_CUDA_SLOT_DENSE 0xFFu

#define VOX_CUDA_CAMERA_SIMPLE 0   /* simple-camera.c: quaternion rotation      */
#define VOX_CUDA_CAMERA_DOOM   1   /* doom-camera.c: yaw + vertical shift k     */

struct vox_node;
typedef struct vox_cuda_tree vox_cuda_tree;

/* The state screen2world reads, for the two camera classes the reference
 * ships (simple-camera.c:10-17, doom-camera.c:8-15). */
typedef struct {
    int32_t kind;
    float position[3];
    float rotation[4];           /* simple: unit quaternion (w, i, j, k)      */
    float mul, xsub, ysub;       /* set_window_size (simple-camera.c:120-136) */
    float sinphi, cosphi, k;     /* doom only                                 */
} vox_cuda_camera;

typedef struct {
    uint64_t nodes;          /* non-NULL nodes                            */
    uint64_t inner;          /* inner nodes                               */
    uint64_t leaves;         /* regular (incl. overflowed) leaves         */
    uint64_t dense_leaves;   /* dense leaves                              */
    uint64_t dots;           /* voxels stored in regular leaves           */
    uint64_t depth;          /* inner nodes on the longest root-leaf path */
    uint64_t device_bytes;   /* bytes of the device pool                  */
} vox_cuda_tree_info;

const char *vox_cuda_strerror(int code);

/* Flatten `root` (any tree built with the reference node layout; NULL is the
 * empty tree) into a device pool on the current device.  The voxel size is
 * read from vox_voxel now and embedded in the pool.  Replaces: nothing in the
 * reference (the reference searches host memory directly). */
int vox_cuda_tree_upload(const struct vox_node *root, vox_cuda_tree **out);
int vox_cuda_tree_free(vox_cuda_tree *tree);
/* Reload a device tree from `root` after the host tree was edited
 * (vox_insert_voxel, vox_delete_voxel; no counterpart in the reference,
 * whose trees live on the host).  Waits for all work on the device first
 * (kernels in flight may read the old image), then flattens `root` again
 * and copies it into the handle's device memory, growing it if needed.
 * Pre-order leaf ids are those of the edited tree afterwards. */
int vox_cuda_tree_refresh(vox_cuda_tree *tree, const struct vox_node *root);
/* Flatten and check `root` on the host only (no device needed) and report
 * what vox_cuda_tree_upload would allocate: the basis of memory budgets.
 * VOX_CUDA_EDEPTH / ETOOBIG as the upload would return them. */
int vox_cuda_tree_measure(const struct vox_node *root, vox_cuda_tree_info *info);
int vox_cuda_tree_get_info(const vox_cuda_tree *tree, vox_cuda_tree_info *info);

/* ---- trees built on the device (tree.c:249-338, datareader.c:11-85) ----
 *
 * The tree vox_make_tree(set, n) would build, node for node and voxel for
 * voxel, built on the GPU straight into a device tree: the image equals
 * vox_make_tree followed by vox_cuda_tree_upload byte for byte, pre-order
 * leaf ids included.  No host tree exists, so vox_cuda_tree_node returns NULL
 * and vox_cuda_tree_node_id fails for these handles; everything else (rays,
 * balls, frames, batches, servers, refresh from a host tree) works as for an
 * uploaded tree.  The voxel size is read from vox_voxel, as by vox_make_tree.
 * Synchronous; n = 0 gives the empty tree.  Sets of 2^31 voxels or more:
 * VOX_CUDA_ETOOBIG. */
/* `set`: n voxels (a vox_dot array, 3n floats) in host memory, left
 * unmodified (vox_make_tree reorders its set). */
int vox_cuda_tree_build(const float *set, size_t n, vox_cuda_tree **out);
/* `d_set`: n voxels (3n floats) in device memory of the current device. */
int vox_cuda_tree_build_device(const float *d_set, size_t n, vox_cuda_tree **out);

/* vox_make_tree builds sets of at least this many voxels on the GPU (when a
 * device is present): the host tree is then made from the device image --
 * node for node the tree of vox_make_tree_host, `set` left in the same order
 * -- and the device copy is kept for the tree's first vox_cuda_tree_upload
 * (single queries and render contexts upload through it), dropped by an edit
 * or vox_destroy_tree.  Default 65536; SIZE_MAX keeps every build on the
 * host.  Returns the previous value. */
size_t vox_cuda_make_tree_gpu_min(size_t n);

/* Which samples are solid.  With mask == NULL: lo <= sample <= hi (the
 * demo's "sample > threshold" is lo = threshold + 1, hi = 0xFFFFFFFF; the
 * engine's ranged reader [min, max) is lo = min, hi = max - 1).  Otherwise
 * bit (sample & 7) of mask[sample >> 3] for samplesize 1 or 2: any predicate
 * of the reference's test block (datareader.h:34), tabulated. */
typedef struct {
    uint32_t lo, hi;
    const uint8_t *mask;
} vox_cuda_raw_test;

/* datareader.c:11-85 with the test on the GPU: `samples` (host memory) holds
 * dim[0] x dim[1] x dim[2] samples of `samplesize` (1..4) little-endian
 * bytes, the last index fastest; the voxel of sample (i, j, k) has its
 * minimum corner at (i, j, k) * vox_voxel, and the set is in that order.
 * Returns the tree of the solid voxels (empty if none, where the reference
 * returns NULL).  Volumes of 2^32 samples or more: VOX_CUDA_ETOOBIG. */
int vox_cuda_tree_build_raw(const void *samples, const unsigned dim[3], unsigned samplesize,
                            const vox_cuda_raw_test *test, vox_cuda_tree **out);
/* vox_read_raw_data (datareader.h:34-37): the file must hold exactly
 * dim[0]*dim[1]*dim[2]*samplesize bytes ("Wrong size of dataset" otherwise);
 * on failure *error (if error is not NULL) is set to a static string. */
int vox_cuda_read_raw_data(const char *filename, const unsigned dim[3], unsigned samplesize,
                           const vox_cuda_raw_test *test, vox_cuda_tree **out, const char **error);

/* The device image of a tree copied to host memory: *n_units 16-byte units
 * (pool_layout.h) and *n_ids pre-order id -> record offset entries.  With
 * NULL buffers only the sizes are reported; buffers smaller than the sizes:
 * VOX_CUDA_EINVAL.  For tests, tools and serialisation. */
int vox_cuda_tree_image(const vox_cuda_tree *tree, void *units, size_t units_cap, uint32_t *rec_of_id,
                        size_t ids_cap, size_t *n_units, size_t *n_ids);
/* The same image made on the host only (no GPU is used): what
 * vox_cuda_tree_upload would copy to the device for `root` at the current
 * vox_voxel.  Sizes and buffers as vox_cuda_tree_image; VOX_CUDA_ETOOBIG when
 * the tree exceeds the image limits. */
int vox_cuda_tree_flatten_host(const struct vox_node *root, void *units, size_t units_cap,
                               uint32_t *rec_of_id, size_t ids_cap, size_t *n_units, size_t *n_ids);

/* ---- vox_dot layouts -------------------------------------------------------
 * A voxvision built with SSE_INTRIN (its default on x86, CMakeLists.txt:19)
 * has a 16-byte vox_dot -- float[4] aligned to 16 bytes -- so its struct
 * vox_box is 32 bytes and its struct vox_node 128 (voxvision.h.in:45-57,
 * tree.h:22-38).  Without SSE_INTRIN vox_dot is float[3] and struct vox_node
 * 112 bytes: the layout include/voxtrees.h declares, the only one on aarch64,
 * and the one the calls above read.  The *_layout calls read a tree of either
 * layout (VOX_CUDA_LAYOUT_*); `voxel` is the voxel size to embed (3 floats,
 * NULL: this library's vox_voxel).  A tree of the SSE layout gives the image,
 * and so every result, that the scalar layout of the same nodes gives;
 * vox_cuda_tree_node returns the caller's own (SSE-layout) nodes.  Replace:
 * nothing in the reference (its searches read its own layout in place). */
#define VOX_CUDA_LAYOUT_SCALAR 0
#define VOX_CUDA_LAYOUT_SSE    1
int vox_cuda_tree_upload_layout(const struct vox_node *root, int layout, const float *voxel, vox_cuda_tree **out);
int vox_cuda_tree_refresh_layout(vox_cuda_tree *tree, const struct vox_node *root, int layout, const float *voxel);
int vox_cuda_tree_flatten_host_layout(const struct vox_node *root, int layout, const float *voxel, void *units,
                                      size_t units_cap, uint32_t *rec_of_id, size_t ids_cap, size_t *n_units,
                                      size_t *n_ids);
/* Code compiled against a voxvision.h with SSE_INTRIN defined (which makes
 * its vox_dot 16 bytes) that includes this header gets the SSE reading under
 * the plain names, with its own vox_voxel, as its voxvision.h picks its
 * vox_dot.  Define VOX_CUDA_KEEP_SCALAR_NAMES to turn this off. */
#if defined(SSE_INTRIN) && !defined(VOX_CUDA_KEEP_SCALAR_NAMES)
#define vox_cuda_tree_upload(root, out) \
    vox_cuda_tree_upload_layout((root), VOX_CUDA_LAYOUT_SSE, vox_voxel, (out))
#define vox_cuda_tree_refresh(tree, root) \
    vox_cuda_tree_refresh_layout((tree), (root), VOX_CUDA_LAYOUT_SSE, vox_voxel)
#define vox_cuda_tree_flatten_host(root, units, units_cap, rec_of_id, ids_cap, n_units, n_ids)             \
    vox_cuda_tree_flatten_host_layout((root), VOX_CUDA_LAYOUT_SSE, vox_voxel, (units), (units_cap), (rec_of_id), \
                                      (ids_cap), (n_units), (n_ids))
#endif

/* The check every upload makes before copying an image (no GPU is used):
 * every offset a search can follow from the root record stays inside the
 * n_units units, every kind is known, leaf ids are below n_nodes, and each of
 * the n_nodes nodes is reached exactly once.  VOX_CUDA_OK or VOX_CUDA_EINVAL. */
int vox_cuda_image_check(const void *units, size_t n_units, size_t n_nodes);
/* Pre-order index -> host node (NULL when out of range). */
const struct vox_node *vox_cuda_tree_node(const vox_cuda_tree *tree, uint32_t id);
/* Host node -> pre-order index; VOX_CUDA_EINVAL when the node is not in the tree. */
int vox_cuda_tree_node_id(const vox_cuda_tree *tree, const struct vox_node *node, uint32_t *id);

/* Ray batch.  origins, dirs: n x 3 floats.  Outputs per ray: leaf_id
 * (pre-order index or VOX_CUDA_MISS), slot (index of the winning voxel in a
 * regular leaf, VOX_CUDA_SLOT_DENSE for a dense leaf or a miss), points
 * (n x 3, written only on a hit, like `res`).  roots: NULL to start every
 * ray at the tree's root, else n pre-order indices of the node each search
 * starts from (vox_ray_tree_intersection accepts any node as its root;
 * renderer.c:297).  slot and points may be NULL.  Batches of 65,536 rays or
 * more are traced grouped by direction and origin (results are the same for
 * any order), with a stream-ordered scratch allocation (cudaMallocAsync) of
 * about 6 bytes per ray for that order.
 * Replaces vox_ray_tree_intersection (src/voxtrees/search.h:24-26). */
int vox_cuda_ray_batch(const vox_cuda_tree *tree, const float *origins, const float *dirs,
                       const uint32_t *roots, size_t n, uint32_t *leaf_id, uint8_t *slot,
                       float *points, void *stream);
int vox_cuda_ray_batch_device(const vox_cuda_tree *tree, const float *origins, const float *dirs,
                              const uint32_t *roots, size_t n, uint32_t *leaf_id, uint8_t *slot,
                              float *points, void *stream);

/* Ball batch.  centres: n x 3 floats, radii: n floats -> hit[i] = 0 / 1.
 * Replaces vox_tree_ball_collidep (src/voxtrees/search.h:36-37). */
int vox_cuda_ball_batch(const vox_cuda_tree *tree, const float *centres, const float *radii,
                        size_t n, uint8_t *hit, void *stream);
int vox_cuda_ball_batch_device(const vox_cuda_tree *tree, const float *centres,
                               const float *radii, size_t n, uint8_t *hit, void *stream);

/* One BEST-quality frame: camera ray generation, search and the colour
 * lookup fused in one kernel, written to a linear w x h ARGB8888 frame
 * (pixel (x, y) at argb[y * w + x]; misses are 0).  texture: the 32^3 u8
 * colour texture (index x*1024 + y*32 + z).  w must be a multiple of 16 and
 * h of 4 (renderer.c:97-100).  vox_cuda_render draws the frame into a
 * device frame the calling thread keeps (w*h*4 bytes, grown as larger frames
 * come, freed when the thread ends); while the kernel runs, a
 * second stream of the calling thread copies zeros into the host frame
 * outside the tree's screen rectangle, and the rectangle follows the kernel
 * (page-locked host frames take the copies at full speed; pageable ones
 * work too).
 * Replaces vox_render + vox_redraw with quality VOX_QUALITY_BEST
 * (src/voxrnd/renderer.c:200-327). */
int vox_cuda_render(const vox_cuda_tree *tree, const vox_cuda_camera *camera,
                    uint32_t w, uint32_t h, const uint8_t *texture, uint32_t *argb,
                    void *stream);
/* n BEST frames of one tree, camera cams[i] into the host buffer frames[i]
 * (w*h ARGB each; the buffers must not overlap, and their contents are
 * undefined until the call returns), with `tex` copied in once: what n calls of
 * vox_cuda_render give, drawn by one persistent launch (up to 1024 frames
 * and 2 GiB of device frames a launch) and each copied out on a second
 * stream as soon as it is complete, while the rest are drawn (for the last
 * four frames of a launch, the zeros outside the tree's screen rectangle
 * are written early and only the rectangle follows); the calling
 * thread waits for each frame's completion (page-locked frames: the copies
 * run asynchronously; pageable ones hold the thread for their copy).  The
 * device frames are kept per thread for later calls.  Returns when all n
 * frames are in host memory; VOX_CUDA_ESTACK if any search overflowed,
 * VOX_CUDA_ETIMEOUT if a frame was not complete within 60 s. */
int vox_cuda_render_frames(const vox_cuda_tree *tree, const vox_cuda_camera *cams, uint32_t n, uint32_t w,
                           uint32_t h, const uint8_t *texture, uint32_t *const *frames, void *stream);
int vox_cuda_render_device(const vox_cuda_tree *tree, const vox_cuda_camera *camera,
                           uint32_t w, uint32_t h, const uint8_t *texture, uint32_t *argb,
                           void *stream);

/* Lights.  A snapshot of a light manager (include/voxrnd.h) on the device;
 * frames drawn with it are coloured as the reference's get_color with a
 * light manager (renderer.c:40-49, lights.c:91-116): ambient light plus the
 * contribution of every light sphere containing the hit, summed in the
 * M-tree's order, min(light, 1) * texel per channel.  Changes to the manager
 * after the upload are not seen: upload again.  M-trees deeper than 9
 * levels: VOX_CUDA_EDEPTH.  No counterpart in the reference beyond the
 * drop-in context (vox_context_set_light_manager), which uses these. */
typedef struct vox_cuda_lights vox_cuda_lights;
struct vox_light_manager;
int vox_cuda_lights_upload(const struct vox_light_manager *light_manager, vox_cuda_lights **out);
int vox_cuda_lights_free(vox_cuda_lights *lights);
/* A frame of any quality lit by `lights` (NULL: grey texels, as
 * vox_cuda_render_quality); host buffers as vox_cuda_render, device
 * buffers as vox_cuda_render_device. */
int vox_cuda_render_lit(const vox_cuda_tree *tree, const vox_cuda_camera *camera, uint32_t w, uint32_t h,
                        unsigned int quality, const uint8_t *texture, const vox_cuda_lights *lights,
                        uint32_t *argb, void *stream);
int vox_cuda_render_lit_device(const vox_cuda_tree *tree, const vox_cuda_camera *camera, uint32_t w, uint32_t h,
                               unsigned int quality, const uint8_t *texture, const vox_cuda_lights *lights,
                               uint32_t *argb, void *stream);
/* A frame through a camera class the device cannot compute (replaces the
 * camera->iface->screen2world calls of vox_render, renderer.c:200-319): the
 * caller gives every pixel's direction in `dirs` (device memory, 3 floats a
 * pixel, rows of w pixels; the camera's screen2world(x, y)) and the camera's
 * position in `origin` (host, 3 floats).  Any quality, FAST and ADAPTIVE as
 * the reference draws them from those directions; BEST traces every pixel
 * from the root.  `lights` may be NULL.  Same geometry rules and errors as
 * vox_cuda_render_lit_device. */
int vox_cuda_render_rays_device(const vox_cuda_tree *tree, const float *origin, const float *dirs, uint32_t w,
                                uint32_t h, unsigned int quality, const uint8_t *texture,
                                const vox_cuda_lights *lights, uint32_t *argb, void *stream);

/* Settings of the BEST-quality frame kernel behind vox_cuda_render*,
 * process-wide (no counterpart in the reference, whose renderer has no
 * kernel).  cull = 1: trace only the rectangle of vox_cuda_frame_rect for the
 * tree's bounding box and clear the rest of the frame; 0: trace every pixel.
 * overlap = 1: launch with programmatic dependent launch, so that a frame's
 * traversal starts while the previous kernel of the stream finishes; the
 * kernel still reads the texture and writes the frame only after that
 * kernel has completed, so stream order holds for all caller memory; 0: an
 * ordinary launch.  Every setting draws the same frame.  Defaults: 1, 1.
 * Values other than 0 and 1: VOX_CUDA_EINVAL. */
typedef struct {
    uint32_t cull;
    uint32_t overlap;
} vox_cuda_render_config;
int vox_cuda_render_set_config(const vox_cuda_render_config *config);
int vox_cuda_render_get_config(vox_cuda_render_config *config);

/* The rectangle [rect[0], rect[2]) x [rect[1], rect[3]) of a w x h frame
 * outside which no pixel's ray can enter the box bbox (min x, y, z, max x,
 * y, z), rounded out to multiples of 8 x 4 pixels; all zero when no pixel
 * can.  The BEST frame kernel traces only this rectangle of the tree's
 * bounding box and clears the rest.  Host-only arithmetic, no GPU needed.
 * No counterpart in the reference, which traces every pixel. */
int vox_cuda_frame_rect(const float *bbox, const vox_cuda_camera *camera, uint32_t w, uint32_t h,
                        uint32_t *rect);

/* Quality values of vox_context_set_quality (src/voxrnd/renderer.h). */
#define VOX_CUDA_QUALITY_BEST                0x0
#define VOX_CUDA_QUALITY_FAST                0x1
#define VOX_CUDA_QUALITY_ADAPTIVE            0x2
#define VOX_CUDA_QUALITY_RAY_MERGE           0x4
#define VOX_CUDA_QUALITY_RAY_MERGE_ACCURATE  0x8
#define VOX_CUDA_QUALITY_RM_MASK             0xC
#define VOX_CUDA_QUALITY_MODE_MASK           0x3

/* One frame in any quality the reference accepts (renderer.c:179-195):
 * BEST runs the per-pixel kernel above; FAST and ADAPTIVE (with or without
 * ray merging) follow each 4x4 square's sequence of renderer.c:215-318 (its
 * Z-order, the previous pixel's leaf as the search root, the corner test),
 * a square on half a warp: every pixel's search from the root, then the
 * searches from the square's leaf for the pixels still to come.  The
 * _device calls allocate nothing; the host-buffer calls draw into the
 * calling thread's device frame and send it to `argb` as vox_cuda_render
 * does.
 * Pixels the reference leaves undrawn are 0.  EINVAL for a combination
 * vox_context_set_quality rejects.
 * Replaces vox_render + vox_redraw (src/voxrnd/renderer.c:200-327). */
int vox_cuda_render_quality(const vox_cuda_tree *tree, const vox_cuda_camera *camera,
                            uint32_t w, uint32_t h, unsigned int quality, const uint8_t *texture,
                            uint32_t *argb, void *stream);
int vox_cuda_render_quality_device(const vox_cuda_tree *tree, const vox_cuda_camera *camera,
                                   uint32_t w, uint32_t h, unsigned int quality,
                                   const uint8_t *texture, uint32_t *argb, void *stream);

/* Work counters of the same searches (no results): counts[0] = nodes whose
 * box was tested, counts[1] = inner nodes entered, counts[2] = voxels
 * tested, summed over the batch or frame (the reference's probes
 * rti__voxels__traversed etc., src/voxtrees/voxtrees-dtrace.d).  counts is a
 * device pointer to 3 uint64 that the call adds to. */
int vox_cuda_render_counts_device(const vox_cuda_tree *tree, const vox_cuda_camera *camera,
                                  uint32_t w, uint32_t h, uint64_t *counts, void *stream);
int vox_cuda_ray_counts_device(const vox_cuda_tree *tree, const float *origins, const float *dirs,
                               size_t n, uint64_t *counts, void *stream);
int vox_cuda_ball_counts_device(const vox_cuda_tree *tree, const float *centres,
                                const float *radii, size_t n, uint64_t *counts, void *stream);

/* ---- Batched frames ------------------------------------------------------
 * Many frames -- cameras of any resolution over any number of resident
 * trees -- drawn by one persistent kernel from a shared work queue and
 * replayed from a CUDA graph.  Each frame is bit-identical to a
 * vox_cuda_render_device call with the same tree, camera and size; the
 * batch only removes the per-frame launch and the per-frame tail.
 * Replaces: a loop of vox_render calls over several contexts
 * (src/voxrnd/renderer.c:200-319), one frame at a time. */
typedef struct {
    const vox_cuda_tree *tree;
    vox_cuda_camera camera;
    uint32_t w, h;               /* w a multiple of 16, h of 4            */
    const uint8_t *texture;      /* device, 32^3 bytes                    */
    uint32_t *argb;              /* device, w * h pixels                  */
} vox_cuda_frame_job;

/* tile_w x tile_h pixels per warp tile: 8x4, 16x2, 32x1 (one ray per thread)
 * or 8x8, 16x4 (two rays per thread); tiles_per_grab: tiles a warp takes
 * from the queue at once (1..64); blocks_per_sm: resident 128-thread blocks
 * per SM (1..16); stack_class: the traversal stack per ray, 0 = the smallest
 * that holds the deepest tree of the batch (28 entries up to depth 9, 64 up
 * to 21, 256 up to 85), 1 or 2 = at least 64 or 256 entries. */
typedef struct {
    uint32_t tile_w, tile_h;
    uint32_t tiles_per_grab;
    uint32_t blocks_per_sm;
    uint32_t stack_class;
} vox_cuda_batch_config;

typedef struct vox_cuda_batch vox_cuda_batch;

/* Build a batch of njobs (1..1024) frames; config NULL = 8x4 tiles, 1 tile
 * per grab, 4 blocks per SM.  The trees, textures and frames must outlive the
 * batch. */
int vox_cuda_batch_create(const vox_cuda_frame_job *jobs, uint32_t njobs,
                          const vox_cuda_batch_config *config, vox_cuda_batch **out);
/* Change one frame's camera; takes effect at the next launch. */
int vox_cuda_batch_set_camera(vox_cuda_batch *batch, uint32_t job, const vox_cuda_camera *camera);
/* Replay the graph on `stream` (asynchronous).  Waits for the batch's
 * previous replay first, so cameras set in between are the ones drawn. */
int vox_cuda_batch_launch(vox_cuda_batch *batch, void *stream);
int vox_cuda_batch_get_config(const vox_cuda_batch *batch, vox_cuda_batch_config *config);
int vox_cuda_batch_set_config(vox_cuda_batch *batch, const vox_cuda_batch_config *config);
/* Time every candidate configuration (reps timed replays each, 0 = 3) on this
 * batch -- tile shapes, tiles per grab, blocks per SM, and the smallest stack
 * class against the next larger one -- keep the fastest and report it
 * (chosen, best_ms may be NULL). */
int vox_cuda_batch_autotune(vox_cuda_batch *batch, void *stream, uint32_t reps,
                            vox_cuda_batch_config *chosen, float *best_ms);
int vox_cuda_batch_free(vox_cuda_batch *batch);

/* Draw njobs frames (1..VOX_CUDA_NOALLOC_MAX_JOBS) like a batch, in one
 * persistent-kernel launch on `stream`, without allocating any memory.  No
 * counterpart in the reference: it is for callers that cannot allocate when
 * they render -- loops that must not stall on cudaMalloc, hosts that own all
 * GPU memory through their own budget, code running with the device nearly
 * full.  Its scratch (job table and work-queue head) is a fixed 16 KiB array
 * in the library's device image, kept by every GPU that loads the library
 * until exit.  Frames are bit-identical to vox_cuda_render_device's.
 * More than VOX_CUDA_NOALLOC_MAX_JOBS jobs: VOX_CUDA_ECAPACITY.  All calls
 * share the array: calls whose work overlaps on the GPU race and must be
 * ordered (same stream, or synchronised).  The job table reaches the GPU as
 * a kernel argument, so the call neither copies from host memory nor waits
 * for earlier work on `stream`.  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) and caches it for the process: make
 * that first call before starting any stream capture, and do not call this
 * after cudaDeviceReset on that device. */
#define VOX_CUDA_NOALLOC_MAX_JOBS 64
int vox_cuda_render_frames_noalloc(const vox_cuda_frame_job *jobs, uint32_t njobs, void *stream);

/* ---- Request server --------------------------------------------------------
 * Frame and ball-collision requests from any number of client threads over
 * resident trees, admitted by memory budgets and batched continuously:
 * everything admitted since the previous launch goes out in the next one, on
 * the next of several streams, so requests that arrive while others run
 * overlap with them on the device.  Frames are drawn into device memory and
 * copied into pinned host memory after their launch's kernel; ball hits are
 * written there in place.  The device budget holds the resident trees, the
 * per-launch job tables (256 bytes per frame) and the frames being drawn
 * (w*h*4 bytes); the pinned-host budget holds each admitted request's result
 * (w*h*4 bytes, or n) and staged ball inputs (16 bytes per ball), in
 * power-of-two size classes from 4 KiB.  Each result equals the plain entry
 * point's for the same request alone.
 * Replaces: applications calling vox_render / vox_tree_ball_collidep from
 * many threads (renderer.h:208 is callable from any thread). */
typedef struct {
    uint64_t budget_bytes;       /* device bytes: resident trees, job tables, frames  */
    uint64_t host_budget_bytes;  /* pinned host bytes for results and staged inputs   */
    uint32_t max_inflight;   /* requests admitted at once                         */
    uint32_t max_batch;      /* requests per launch (1..1024)                     */
    uint32_t streams;        /* launch streams (1..32)                            */
    uint32_t max_launches;   /* launches in flight at once                        */
    uint32_t frames_on_device;  /* 0: frames are copied into pinned host memory;
                                   1: frames stay in device memory the server
                                   owns (vox_cuda_server_result gives a device
                                   pointer; the frame holds its share of the
                                   device budget until released) -- for clients
                                   that use the frames on the GPU */
} vox_cuda_server_config;

typedef struct {
    uint64_t submitted, completed, rejected, launches;
    uint64_t bytes_in_use, peak_bytes;            /* device budget */
    uint64_t pending, inflight;
    uint64_t host_bytes_in_use, host_peak_bytes;  /* pinned-host budget */
    /* where the worker thread's time goes (ns since creation): all of its
     * work outside its waits; building and enqueueing launches; pinning new
     * host result buffers (host_pins of them: the pool's misses); device
     * allocations of job tables and frames.  frame_bytes_out: frame bytes
     * copied to host memory; frame_bytes_full: the bytes of those frames
     * (w*h*4 each) -- a result buffer the server reuses already holds zeros
     * outside the rectangle of the frame it held last, so only the part of a
     * frame that can differ is copied.  host_slabs: 128 MiB slabs pinned for
     * results, at creation and by the server's refill thread. */
    uint64_t worker_busy_ns, build_ns, host_pin_ns, host_pins, device_alloc_ns, frame_bytes_out, host_slabs;
    uint64_t frame_bytes_full;
} vox_cuda_server_stats;

typedef struct vox_cuda_server vox_cuda_server;

/* config NULL = 40 GiB device budget, 16 GiB pinned host budget, 256 in
 * flight, 32 per launch, 16 streams, 32 launches in flight, frames copied to
 * host memory.  texture: host 32^3 bytes used for every frame.  Half the
 * pinned-host budget (at most 8 GiB; with frames_on_device an eighth, at most
 * 1 GiB) is page-locked here, in 128 MiB slabs that results are carved from
 * (about 0.6 s for 8 GiB); a thread of the server keeps two more slabs pinned
 * ahead of need, up to the budget. */
int vox_cuda_server_create(const vox_cuda_server_config *config, const uint8_t *texture,
                           vox_cuda_server **out);
/* Make a tree available to requests (charged to the budget while the server
 * lives; the tree must outlive the server). */
int vox_cuda_server_add_tree(vox_cuda_server *srv, const vox_cuda_tree *tree, uint32_t *tree_id);
/* Queue a BEST frame / a ball batch (inputs are copied); the ticket names the
 * request.  VOX_CUDA_EBUDGET if it could never fit the budget. */
int vox_cuda_server_submit_frame(vox_cuda_server *srv, uint32_t tree_id, const vox_cuda_camera *camera,
                                 uint32_t w, uint32_t h, uint64_t *ticket);
int vox_cuda_server_submit_balls(vox_cuda_server *srv, uint32_t tree_id, const float *centres,
                                 const float *radii, uint32_t n, uint64_t *ticket);
/* Wait up to timeout_ms for a request: its status, or VOX_CUDA_ETIMEOUT. */
int vox_cuda_server_wait(vox_cuda_server *srv, uint64_t ticket, uint32_t timeout_ms);
/* A finished request's result (w*h ARGB pixels, or n hit bytes) in server
 * memory -- pinned host memory, or for frames of a server with
 * frames_on_device set, device memory of the server's device -- valid until
 * vox_cuda_server_release and read-only: the server reuses a host frame's
 * buffer and copies into it only what differs from the frame it held last.
 * times_ns (may be NULL) gets submission, launch and completion times
 * (steady clock, ns). */
int vox_cuda_server_result(vox_cuda_server *srv, uint64_t ticket, const void **data, size_t *bytes,
                           uint64_t *times_ns);
int vox_cuda_server_release(vox_cuda_server *srv, uint64_t ticket);
int vox_cuda_server_get_stats(vox_cuda_server *srv, vox_cuda_server_stats *stats);
/* Finish all queued requests, then stop. */
int vox_cuda_server_destroy(vox_cuda_server *srv);

/* Host-side fault injection, for tests of the server's failure handling (no
 * GPU fault is made; the reference has no counterpart).  The fault hits the
 * next launch the server builds:
 *   VOX_CUDA_INJECT_REQUEST_ERROR: its requests end with VOX_CUDA_ECUDA, as if
 *     their enqueue had failed; later requests are served as usual.
 *   VOX_CUDA_INJECT_WORKER_FAILURE: building it throws an allocation failure
 *     in the server's worker.  The worker waits for the launches in flight
 *     (their requests keep their results), ends every other request with
 *     VOX_CUDA_ENOMEM and stops; later submissions return VOX_CUDA_ENOMEM and
 *     vox_cuda_server_destroy still frees everything.  A real allocation
 *     failure in the worker takes the same path. */
#define VOX_CUDA_INJECT_REQUEST_ERROR  1
#define VOX_CUDA_INJECT_WORKER_FAILURE 2
int vox_cuda_server_inject(vox_cuda_server *srv, int what);

/* Replay a request trace against a server, for capacity measurements (no
 * counterpart in the reference).  Requests are submitted from the calling
 * thread at their arrival times (seconds after the call starts, ascending);
 * `collectors` threads (1..64) wait for them in arrival order, record the
 * server's submission, launch and completion times and release them.
 * Returns when every request has completed (out[i].status is its status;
 * a submission refused by the server keeps that error). */
typedef struct {
    uint32_t kind;               /* 0 BEST frame, 1 ball batch          */
    uint32_t tree_id;
    vox_cuda_camera camera;      /* frame                               */
    uint32_t w, h;               /* frame                               */
    const float *centres;        /* ball batch, n x 3 (host)            */
    const float *radii;          /* ball batch, n (host)                */
    uint32_t n;                  /* ball batch                          */
    double arrival_s;
} vox_cuda_replay_request;

typedef struct {
    int32_t status;
    uint64_t submit_ns, launch_ns, done_ns;
} vox_cuda_replay_result;

int vox_cuda_server_replay(vox_cuda_server *srv, const vox_cuda_replay_request *requests, uint32_t n,
                           uint32_t collectors, vox_cuda_replay_result *results);

/* Library version and the number of kernel launches made so far by this
 * process (all entry points); used to report launch counts. */
const char *vox_cuda_version(void);
uint64_t vox_cuda_launch_count(void);

/* Measurement aid, no counterpart in the reference: the L2 read bandwidth of
 * the current device in GB/s, from one kernel that reads a `bytes` buffer
 * (small enough to stay in L2, e.g. 32 MiB) `reps` times over with loads that
 * bypass L1, timed with CUDA events after a warm pass.  The roofline of the
 * search kernels, whose tree mostly stays in L2, is set against it.
 * Allocates and frees the buffer itself. */
int vox_cuda_measure_l2_read(size_t bytes, uint32_t reps, float *gbs);

/* 1 in the checked build (libvoxtrees_cuda_checked.so, compiled with
 * -DVOX_CUDA_CHECKED): every search load first checks its index against the
 * uploaded tree and light arrays, and a search that meets an index outside
 * them ends with VOX_CUDA_ERANGE instead of reading; 0 in the normal build,
 * which relies on the upload-time validation of the tree image. */
int vox_cuda_build_checked(void);

#ifdef __cplusplus
}
#endif
#endif
