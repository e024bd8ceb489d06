// dr_internal.h - accessors shared between the library's host translation units (not exported).
#pragma once
#include "../../include/dr_api.h"
#include "dr_device.cuh"

// Device-side view of a scene (pointers into the scene's own device buffers).
const drd::Scene *dr_internal_scene_device(const dr_scene *scene);

// True when every texture the scene's materials use has been set (dr_scene_set_textures).
bool dr_internal_scene_textures_ok(const dr_scene *scene);

// Records the message returned by dr_last_error() on this thread.
void dr_internal_set_error(const char *msg);
