// Host-to-device copies of many caller arrays through a page-locked staging ring.
#pragma once
#include <vector>

#include "common.cuh"

namespace jues {

// one contiguous range, copied from src to dst
struct HostSeg {
    void *dst;
    const void *src;
    size_t bytes;
};

// Host -> device (src host, dst device), in order on ctx->stream.  Host threads fill 64 MB
// page-locked slots (three in a ring, allocated once per context) while the link drains the
// previous slot, so no caller memory is page-locked: registering memory costs about a
// millisecond per call, which is most of the time for hundreds of small arrays.  Returns after
// the last copy is queued; a slot is refilled only once its copies have finished.
void staged_h2d(Ctx *ctx, const std::vector<HostSeg> &segs);

// Device -> host (src device, dst host) after the work queued on ctx->stream; returns with the
// data in the caller's arrays.
void staged_d2h(Ctx *ctx, const std::vector<HostSeg> &segs);

// releases the ring and its threads (context destruction)
void staging_destroy(Staging *st);

}  // namespace jues
