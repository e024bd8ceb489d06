// ref_driver.h - what oracle/ref_driver.cu shares with other code compiled against the reference
// sources (the GB300Renderer test harness): the scene object behind dref_scene_create and the
// record-to-object constructors.  Test infrastructure only.
#pragma once
#include "DataStructures/Renderers/DumbRenderer/DumbRenderer.cuh"

// A reference scene (geometry octree, materials, lights, textures) and its camera, as the
// reference's DumbRenderer takes them (DumbRenderer.cuh:10-11).
struct RefScene {
	TriScene scene;
	DumbRenderer::CameraManager camera;
};

// Material / light from the flat records documented in ref_driver.cu, through the reference's
// own constructors.
void ref_material(Material<BakedTriFace> &dst, const float *m);
void ref_light(Light &dst, const float *l);
