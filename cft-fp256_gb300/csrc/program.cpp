// program.cpp - the sequencer's host side (placeholder until the GPU
// executor lands): every program entry point refuses by name.
#include "api_core.h"

using namespace cftg;

extern "C" cft_status cft_program_load(cft_device *, const void *, size_t, cft_program **out)
{
    clear_error();
    if (out) *out = nullptr;
    set_error("cft_program_load: the sequencer is not built into this library yet");
    return CFT_ERR_UNSUPPORTED;
}
extern "C" void cft_program_free(cft_program *) {}
extern "C" cft_status cft_program_get_info(cft_program *, cft_program_info *)
{
    clear_error();
    return CFT_ERR_INVALID_ARGUMENT;
}
extern "C" cft_status cft_program_run(cft_program *, const void *, const void *, const void *,
                                      void *, uint32_t *, size_t, uint32_t *, uint32_t *)
{
    clear_error();
    return CFT_ERR_INVALID_ARGUMENT;
}
extern "C" cft_status cft_program_run_bank(cft_program *, const void *, size_t, const void *,
                                           const void *, const void *, void *, uint32_t *,
                                           size_t, uint32_t *, uint32_t *)
{
    clear_error();
    return CFT_ERR_INVALID_ARGUMENT;
}
extern "C" cft_status cft_program_run_ex(cft_program *, const cft_run_args *)
{
    clear_error();
    return CFT_ERR_INVALID_ARGUMENT;
}
extern "C" cft_status cft_program_digest(cft_program *, const void *, size_t, uint8_t *)
{
    clear_error();
    return CFT_ERR_INVALID_ARGUMENT;
}
extern "C" cft_status cft_sha256(const void *, size_t, uint8_t *)
{
    clear_error();
    return CFT_ERR_UNSUPPORTED;
}
