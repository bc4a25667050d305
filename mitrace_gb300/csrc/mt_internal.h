// mt_internal.h - accessors to handle internals for other translation units of
// the library (not part of the public ABI).
#pragma once

#include <cstdint>
#include <string>

#include "../../include/mitrace_gpu.h"

namespace mt {

struct DevScene;

// The handle's uploaded scene and render settings, or nullptr for a null handle.
const DevScene* internal_scene(const mt_handle* h);
// True while an asynchronous render (mt_start) is running on the handle.
bool internal_busy(const mt_handle* h);
// Adds n camera samples to the counter mt_get_stats reports.
void internal_count_samples(mt_handle* h, uint64_t n);
// Records msg as the calling thread's mt_last_error() and returns code.
mt_status internal_error(mt_status code, const std::string& msg);

}  // namespace mt
