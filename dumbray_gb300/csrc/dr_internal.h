// dr_internal.h - accessors shared between the library's host translation units (not exported).
#pragma once
#include "../../include/dr_api.h"
#include "dr_device.cuh"
#include "dr_kernels.h"

// Device-side view of a scene (pointers into the scene's own device buffers).
const drd::Scene *dr_internal_scene_device(const dr_scene *scene);

// True when every texture the scene's materials use has been set (dr_scene_set_textures).
bool dr_internal_scene_textures_ok(const dr_scene *scene);

// Records the message returned by dr_last_error() on this thread.
void dr_internal_set_error(const char *msg);

// Validates one render job (scene, camera, frame buffer, block range, parameters; `who` prefixes
// the error message) and fills its job record: lens focal factor, pixel size by boxing mode,
// sub-pixel steps, sample base and blend weight of the iteration.  Every entry point that renders
// blocks builds its jobs through this one function.
dr_status dr_internal_make_item(const dr_scene *sc, const dr_camera *cam, float *fb, int32_t start_block,
                                int32_t end_block, const dr_render_params *p, const char *who, drk::Item &I);
