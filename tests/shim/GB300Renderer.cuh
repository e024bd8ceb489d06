// GB300Renderer.cuh - the reference-side drop-in for DumbRenderer: the same BlockRenderer plug
// (renderBlocksGPU, __source__/DataStructures/Renderers/BlockRenderer/BlockRenderer.cuh:43-44), with
// the work done by libdumbray_gb300 through its C ABI (include/dr_api.h).
//
// A DumbRay maintainer adds these two files under __source__/DataStructures/Renderers/GB300Renderer/
// and constructs a GB300Renderer wherever a DumbRenderer is constructed (same constructor, same
// setters: scene, camera, boxing mode, bounce limit, samples per pixel, backface culling).  Here the
// files are compiled against the reference sources by tests/shim/build_shim.sh and exercised by the
// shim tests.
//
// What changes against DumbRenderer (DumbRenderer.cu:87-113):
//   * GPU worker threads render their block ranges with dr_render_blocks in the reference-semantics
//     mode (DR_MODE_REFERENCE) into the same device BlockBasedFrameBuffer<8,16> the reference kernel
//     writes; the reference's own BlockRenderer hands out the block ranges, keeps the streams and
//     moves blocks between host and device as before.
//   * The scene is converted once (per TriScene object) into a dr_scene shared by every worker
//     thread: triangles, normals, texture corners and material ids in octree push order, the
//     materials, lights and textures through their stored state.  The camera is converted on every
//     call (it may move between iterations).  Each worker thread (Info::globalThreadId) owns a
//     dr_renderer (wavefront scratch), as each owns a DeviceBlockManager in the reference.
//   * No CPU fallback on the GPU path: a failed call returns false (the message is kept for
//     lastError()), which makes BlockRenderer stop that device's work for the iteration
//     (BlockRenderer.cu:87-92).  CPU worker threads still run the reference's renderBlocksCPU.
//   * Random numbers: the library's counter-based generator keyed by (seed, pixel, sample, bounce),
//     the iteration selecting the samples, in place of DumbRand's per-thread XORWOW state.
#pragma once
#include <mutex>
#include <string>
#include <vector>

#include "DataStructures/Renderers/DumbRenderer/DumbRenderer.cuh"
#include "dr_api.h"

class GB300Renderer : public DumbRenderer {
public:
	GB300Renderer(
		const ThreadConfiguration &configuration = ThreadConfiguration(ThreadConfiguration::ALL, 2),
		const BlockConfiguration &blockSettings = BlockConfiguration(),
		FrameBufferManager *buffer = NULL,
		SceneType *scene = NULL,
		CameraManager *camera = NULL,
		BoxingMode boxingMode = BOXING_MODE_HEIGHT_BASED,
		int maxBounces = 2,
		int samplesPerPixelX = 1,
		int samplesPerPixelY = 1,
		int pixelsPerGPUThread = 1,
		bool ignoreBackfaces = true);
	virtual ~GB300Renderer();

	// Seed of the counter-based random numbers (default 0); each iteration takes new samples.
	void setSeed(uint32_t seed);
	// Message of the last failed GPU call (empty when none failed).
	std::string lastError();
	// Drops the converted scene so that the next render converts getScene() again (after the host
	// changed the scene's geometry, materials, lights or textures).
	void invalidateScene();
	// Octree padding of the converted scene: false (default) the reference's 1.28e-3, so every cast
	// equals Octree::cast bit for bit; true the library's physical-mode padding (2^-18 x the largest
	// coordinate), which holds fewer duplicated triangles per leaf and renders faster, with the same
	// closest hits up to float32 near-ties (two triangles a few ulps apart along the ray).
	void setTightOctree(bool tight);

protected:
	bool renderBlocksGPU(const Info &info, FrameBuffer *host, FrameBuffer *device,
	                     int startBlock, int endBlock, cudaStream_t &renderStream) override;

	// The library call behind renderBlocksGPU, on the device pixels of a block-major frame buffer.
	bool renderDeviceBlocks(int threadSlot, float *deviceBlocks, int width, int height,
	                        int startBlock, int endBlock, cudaStream_t stream);
	// getCamera() as a dr_camera: the lens's stored state (focal factor, segment angles) and the
	// transform's direction basis and point-transform rows.
	bool toCamera(dr_camera &out, std::string &error);

private:
	bool ensureScene(std::string &error);        // sceneLock held
	bool threadRenderer(int slot, dr_renderer **out, std::string &error);
	void fail(const std::string &message);

	std::mutex sceneLock;
	dr_scene *scene;
	const SceneType *converted;                  // the TriScene that `scene` was made from
	std::vector<dr_renderer *> renderers;        // by Info::globalThreadId
	uint32_t seed;
	bool tightOctree;
	std::string error;
};
