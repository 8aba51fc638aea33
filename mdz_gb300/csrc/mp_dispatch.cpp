// Dispatch of the multi-limb kernel by word count.
#include "internal.h"

namespace mdz {

bool mp_words_supported(int words)
{
#define MDZ_CASE(n) \
    if (words == n) \
        return true;
    MDZ_MP_WORDS_LIST(MDZ_CASE)
#undef MDZ_CASE
    return false;
}

int launch_mp(mdzgpu_ctx* ctx, const MpLaunch& p, cudaStream_t s)
{
    switch (p.words) {
#define MDZ_CASE(n) \
    case n:         \
        return launch_words<n>(ctx, p, s);
        MDZ_MP_WORDS_LIST(MDZ_CASE)
#undef MDZ_CASE
    default:
        set_error("mp kernel: %d words not built", p.words);
        return MDZGPU_ERR_UNSUPPORTED;
    }
}

}  // namespace mdz
