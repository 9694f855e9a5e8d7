// svo.cu -- one-bit SVO build and traversal (placeholder entry points).
#include "tgx_internal.cuh"

extern "C" tgx_status tgx_svo_build(tgx_ctx*, const tgx_scene*, const float*, uint32_t, tgx_svo** out)
{
    if (out) *out = nullptr;
    tgx_set_error("tgx_svo_build: not built yet");
    return TGX_ERR_NOT_SUPPORTED;
}
extern "C" void tgx_svo_destroy(tgx_ctx*, tgx_svo*) {}
extern "C" tgx_status tgx_svo_get_info(tgx_ctx*, const tgx_svo*, tgx_svo_info*) { return TGX_ERR_NOT_SUPPORTED; }
extern "C" tgx_status tgx_svo_download(tgx_ctx*, const tgx_svo*, int32_t*, uint32_t*, uint32_t, uint32_t*) { return TGX_ERR_NOT_SUPPORTED; }
extern "C" tgx_status tgx_svo_trace(tgx_ctx*, const tgx_svo*, uint32_t, const float*, const float*, uint32_t, float*, int32_t*) { return TGX_ERR_NOT_SUPPORTED; }
