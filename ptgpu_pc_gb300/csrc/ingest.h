// ingest.h -- scene ingestion from the compact (segment) form straight into
// device shape and light arrays (ingest.cu).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "devbuf.h"
#include "host.h"
#include "types.h"

namespace ptgpu {

// Device room for one model's vertices and indices, reused across calls.
struct IngestScratch {
    DevBuf v, tri;
    std::vector<std::vector<LightRec>> host_lights;   // light records in flight
    void release() { v.release(); tri.release(); host_lights.clear(); }
};

// SampleLights' emitter count for the scene: its emitting shapes, at most
// light_cnt of them (make_lights' rule).
uint32_t compact_light_count(const CompactScene &sc);
bool compact_all_triangles(const CompactScene &sc);
// Writes the scene's count() shapes to d_shapes and its compact_light_count()
// light records to d_lights; returns after the stream has finished them.
cudaError_t ingest_compact(const CompactScene &sc, ptgpu_shape *d_shapes, LightRec *d_lights,
                           IngestScratch &scr, cudaStream_t s);

}  // namespace ptgpu
