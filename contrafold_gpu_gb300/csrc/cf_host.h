// cf_host.h -- what the engine's host translation unit (cf_engine.cu) lends to
// the other host-side translation units: read access to an engine's device,
// stream and float32 parameter blob, its shared-memory opt-in, and the
// thread-local error message behind cf_last_error().
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

struct cf_engine;

namespace cf {

int engine_device(const cf_engine* e);
cudaStream_t engine_stream(const cf_engine* e);
const float* engine_blob32(const cf_engine* e);
// Raises the dynamic shared-memory limit of every engine kernel to `bytes`
// (never lowers it); CF_EINVAL when the device cannot give that much.
int engine_ensure_smem(cf_engine* e, size_t bytes);
// Records `msg` for cf_last_error() and returns `code`.
int engine_fail(int code, const char* msg);

}  // namespace cf
