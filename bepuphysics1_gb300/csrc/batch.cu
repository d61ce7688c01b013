// Batched stepping of many scenes (bepugpu_batch_step).
#include "bepugpu_internal.h"

using namespace bepugpu;

extern "C" bepugpu_status bepugpu_batch_step(bepugpu_context* c, const int32_t* scenes, uint32_t count, float dt,
                                             uint32_t steps, uint32_t flags) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    (void)scenes; (void)count; (void)dt; (void)steps; (void)flags;
    ctx->SetError("batched stepping is not available in this build");
    return BEPUGPU_INVALID_OPERATION;
}
