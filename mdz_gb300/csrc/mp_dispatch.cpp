// Dispatch of the multi-limb kernel by word count.
#include "internal.h"
#include "serve.h"

namespace mdz {

bool mp_words_supported(int words)
{
#define MDZ_CASE(n) \
    if (words == n) \
        return true;
    MDZ_MP_WORDS_LIST(MDZ_CASE)
#undef MDZ_CASE
#define MDZ_CASE(n, g, q) \
    if (words == n)       \
        return true;
    MDZ_MPW_LIST(MDZ_CASE)
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
#define MDZ_CASE(n, g, q) \
    case n:               \
        return launch_wide<g, q>(ctx, p, s);
        MDZ_MPW_LIST(MDZ_CASE)
#undef MDZ_CASE
    default:
        set_error("mp kernel: %d words not built", p.words);
        return MDZGPU_ERR_UNSUPPORTED;
    }
}

int preload_mp_kernels()
{
    int rc = MDZGPU_OK;
#define MDZ_CASE(n)              \
    if (!rc)                     \
        rc = preload_words<n>();
    MDZ_MP_WORDS_LIST(MDZ_CASE)
#undef MDZ_CASE
#define MDZ_CASE(n, g, q)           \
    if (!rc)                        \
        rc = preload_wide<g, q>();
    MDZ_MPW_LIST(MDZ_CASE)
#undef MDZ_CASE
    return rc;
}

// Class kServePerturbClasses + k of the serving engine is the (k+1)-th word
// count of the list.
int serve_mp_class_words(int cls)
{
    int k = kServePerturbClasses - 1;
#define MDZ_CASE(n)      \
    if (++k == cls)      \
        return n;
    MDZ_MP_WORDS_LIST(MDZ_CASE)
#undef MDZ_CASE
    return 0;
}

int launch_serve_mp(ServeDev* d, int mp_class, int num_sms, cudaStream_t s)
{
    switch (serve_mp_class_words(mp_class)) {
#define MDZ_CASE(n) \
    case n:         \
        return launch_serve_mp_words<n>(d, mp_class, num_sms, s);
        MDZ_MP_WORDS_LIST(MDZ_CASE)
#undef MDZ_CASE
    default:
        set_error("serve: method class %d has no multi-limb kernel", mp_class);
        return MDZGPU_ERR_UNSUPPORTED;
    }
}

}  // namespace mdz
