// Internal accessors of swr_context (defined in swr_capi.cu) for entry points that live in
// other translation units.
#pragma once
#include <stdint.h>

struct swr_context;

namespace swr {
// Device status words of the context (reported and reset by swr_finish).
uint32_t* context_status(swr_context* c);
// Counts kernel launches toward swr_stats.launches.
void context_add_launches(swr_context* c, uint64_t n);
}  // namespace swr
