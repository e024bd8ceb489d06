// shim_driver.cu - C ABI around GB300Renderer for the shim tests (test infrastructure only).
//
// The harness drives the drop-in the way BlockRenderer::iterateGPU does (BlockRenderer.cu:74-97):
// renderBlocksGPU(info, host, device, startBlock, endBlock, renderStream) with a host frame buffer
// (FrameBufferManager holding a BlockBuffer) and a device replica of it.  The replica is set up
// with the reference's own host-side steps - TypeTools<BlockBuffer>::prepareForCpyLoad allocates
// the device pixels and registers the mirror (BlockBasedFrameBuffer.impl.cuh:248-279), and the
// device FrameBuffer handle is written as Generic's upload would leave it - but without the
// reference's device-side function-pack set-up (Generic.impl.cuh:195-205 launches a kernel of the
// reference to store device function pointers, which GB300Renderer never calls), so no reference
// kernel runs.  Pixels come back through the reference's FrameBuffer::updateHostBlocks.
#include <cstring>
#include <string>

#include "GB300Renderer.cuh"
#include "ref_driver.h"
#include "DataStructures/Screen/FrameBuffer/BlockBasedFrameBuffer/BlockBasedFrameBuffer.cuh"

namespace {

struct GenericData {
	typedef volatile void *Generic<FrameBufferFunctionPack>::*type;
};
template <class Key>
struct Slot {
	static typename Key::type ptr;
};
template <class Key>
typename Key::type Slot<Key>::ptr;
template <class Key, typename Key::type P>
struct Fill {
	struct Run {
		Run() { Slot<Key>::ptr = P; }
	};
	static Run run;
};
template <class Key, typename Key::type P>
typename Fill<Key, P>::Run Fill<Key, P>::run;
template struct Fill<GenericData, &Generic<FrameBufferFunctionPack>::dataPointer>;

// GB300Renderer with the BlockRenderer entry point and a worker's Info reachable from here.
class Harness : public GB300Renderer {
public:
	using GB300Renderer::GB300Renderer;
	bool render(int slot, FrameBuffer *host, FrameBuffer *device, int start, int end, cudaStream_t stream) {
		Info info;
		std::memset(&info, 0, sizeof(info));
		info.device = 0;
		info.numDeviceThreads = 8;
		info.deviceThreadId = slot;
		info.globalThreadId = slot;
		info.manageSharedData = (slot == 0);
		return renderBlocksGPU(info, host, device, start, end, stream);
	}
	using GB300Renderer::toCamera;
};

struct Frame {
	FrameBufferManager fb;
	BlockBuffer *device_buffer = NULL;     // device BlockBuffer object
	FrameBuffer *device_handle = NULL;     // device FrameBuffer (Generic) handle
	alignas(16) char clone[sizeof(BlockBuffer)];
	bool registered = false;
	Harness *renderer = NULL;
	std::string error;
};

}  // namespace

extern "C" {

// A width x height BlockBuffer frame (host and device replica, device pixels copied from the
// zeroed host pixels) and a GB300Renderer over the reference scene `ref_scene` (dref_scene_create)
// with DumbRenderer's settings.  NULL on failure.
void *dshim_create(void *ref_scene, int width, int height, int fsaa_x, int fsaa_y, int max_bounces, int cull,
                   int boxing, unsigned seed) {
	RefScene *s = (RefScene *)ref_scene;
	Frame *f = new Frame();
	f->fb.cpuHandle()->use<BlockBuffer>();
	if (!f->fb.cpuHandle()->setResolution(width, height)) { delete f; return NULL; }
	BlockBuffer *host = f->fb.cpuHandle()->getObject<BlockBuffer>();
	bool ok = cudaMalloc((void **)&f->device_buffer, sizeof(BlockBuffer)) == cudaSuccess &&
	          cudaMalloc((void **)&f->device_handle, sizeof(FrameBuffer)) == cudaSuccess;
	if (ok) {
		ok = TypeTools<BlockBuffer>::prepareForCpyLoad(host, (BlockBuffer *)f->clone, f->device_buffer, 1);
		f->registered = ok;
	}
	if (ok) ok = cudaMemcpy(f->device_buffer, f->clone, sizeof(BlockBuffer), cudaMemcpyHostToDevice) == cudaSuccess;
	if (ok) {
		alignas(16) char handle[sizeof(FrameBuffer)];
		std::memset(handle, 0, sizeof(handle));
		((Generic<FrameBufferFunctionPack> *)handle)->*Slot<GenericData>::ptr = f->device_buffer;
		ok = cudaMemcpy(f->device_handle, handle, sizeof(handle), cudaMemcpyHostToDevice) == cudaSuccess;
	}
	if (ok) {
		f->renderer = new Harness(Renderer::ThreadConfiguration::cpuOnly(1), BlockRenderer::BlockConfiguration(), &f->fb,
		                          &s->scene, &s->camera, (DumbRenderer::BoxingMode)boxing, max_bounces, fsaa_x, fsaa_y, 1,
		                          cull != 0);
		f->renderer->setSeed(seed);
	}
	if (!ok) {
		if (f->registered) TypeTools<BlockBuffer>::undoCpyLoadPreparations(host, (BlockBuffer *)f->clone, f->device_buffer, 1);
		cudaFree(f->device_buffer);
		cudaFree(f->device_handle);
		delete f;
		return NULL;
	}
	return f;
}

// renderBlocksGPU of worker slot `slot` on blocks [start, end) in `stream`: 1 = rendered.
int dshim_render(void *h, int slot, int start, int end, void *stream) {
	Frame *f = (Frame *)h;
	cudaStream_t s = (cudaStream_t)stream;
	const bool ok = f->renderer->render(slot, f->fb.cpuHandle(), f->device_handle, start, end, s);
	if (!ok) f->error = f->renderer->lastError();
	return ok ? 1 : 0;
}

// Copies blocks [start, end) of the device replica to the host buffer (the reference's
// updateHostBlocks) and writes the whole host buffer block-major (float4 per pixel, blocks of
// 8 x 16) to out.  1 = ok.
int dshim_read(void *h, int start, int end, float *out) {
	Frame *f = (Frame *)h;
	FrameBuffer *host = f->fb.cpuHandle();
	cudaStream_t s = NULL;
	if (cudaStreamCreate(&s) != cudaSuccess) return 0;
	const bool ok = host->updateHostBlocks(f->device_handle, start, end, &s) && cudaStreamSynchronize(s) == cudaSuccess;
	cudaStreamDestroy(s);
	if (!ok) return 0;
	const int blocks = host->getBlockCount(), size = host->getBlockSize();
	for (int b = 0; b < blocks; b++)
		for (int p = 0; p < size; p++) {
			const Color c = host->getBlockPixelColor(b, p);
			float *o = out + 4 * ((size_t)b * size + p);
			o[0] = c.r; o[1] = c.g; o[2] = c.b; o[3] = c.a;
		}
	return 1;
}

// GB300Renderer::setTightOctree.
void dshim_set_tight_octree(void *h, int tight) { ((Frame *)h)->renderer->setTightOctree(tight != 0); }

// The camera GB300Renderer hands the library (1 = ok).
int dshim_camera(void *h, dr_camera *out) {
	Frame *f = (Frame *)h;
	return f->renderer->toCamera(*out, f->error) ? 1 : 0;
}

const char *dshim_error(void *h) { return ((Frame *)h)->error.c_str(); }

void dshim_destroy(void *h) {
	Frame *f = (Frame *)h;
	delete f->renderer;
	BlockBuffer *host = f->fb.cpuHandle()->getObject<BlockBuffer>();
	if (f->registered) TypeTools<BlockBuffer>::undoCpyLoadPreparations(host, (BlockBuffer *)f->clone, f->device_buffer, 1);
	cudaFree(f->device_buffer);
	cudaFree(f->device_handle);
	delete f;
}

}  // extern "C"
