/*
 * frame_memo.h -- what a frame buffer owned by a renderer context still holds
 * from its last frame, so that the next frame clears only part of it (host
 * code; shared by voxtrees_cuda.cu and renderer.cpp, not part of the C ABI).
 */
#ifndef VOX_FRAME_MEMO_H
#define VOX_FRAME_MEMO_H

#include <cuda_runtime_api.h>

#include <cstdint>

#include "../../include/voxtrees_cuda.h"

namespace vox {

/* With `valid`, every pixel of the buffer outside [x0, x1) x [y0, y1) is
 * zero: the traced rectangle of the last frame this library drew into it
 * (its frame kernels write every pixel of that rectangle, and clear the rest
 * of what may hold anything). */
struct FrameMemo {
    bool valid;
    uint32_t x0, y0, x1, y1;
};

}  // namespace vox

/* One frame of any quality into argb (device-addressable), as
 * vox_cuda_render_lit_device does or, with dirs (device memory, 3 floats a
 * pixel), as vox_cuda_render_rays_device does from cam->position.  With a
 * memo, the frame outside its traced rectangle is cleared only where the
 * memo says it may be non-zero, and the memo is updated for the next frame
 * (left invalid when the launch fails; unchanged when the call is refused
 * before anything is written). */
int render_frame_memo(const vox_cuda_tree *t, const vox_cuda_camera *cam, const float *dirs, uint32_t w, uint32_t h,
                      unsigned int quality, const uint8_t *tex, const vox_cuda_lights *lights, uint32_t *argb,
                      cudaStream_t s, vox::FrameMemo *memo);

#endif
