// Unmangled entry points over the reference's volrendjax::* functions (declared in its
// lib/impl/volrend.h:121-175), for loading with ctypes.  Each forwards the XLA custom-call
// arguments unchanged and turns the reference's C++ exception (CUDA_CHECK_THROW, volrend.h:9-16;
// a bad opaque length, serde.h) into a non-zero return, with the message kept for
// ref_last_error().
#include <cstdio>
#include <exception>

#include "volrend.h"

namespace {
thread_local char g_err[512] = "";

template <class F>
int guarded(F &&f) {
    try {
        f();
        g_err[0] = '\0';
        return 0;
    } catch (const std::exception &e) {
        std::snprintf(g_err, sizeof(g_err), "%s", e.what());
        return 1;
    }
}
}  // namespace

#define REF_ENTRY(name)                                                                          \
    extern "C" int ref_##name(cudaStream_t s, void **b, const char *o, std::size_t n) {          \
        return guarded([&] { volrendjax::name(s, b, o, n); });                                   \
    }

REF_ENTRY(pack_density_into_bits)
REF_ENTRY(march_rays)
REF_ENTRY(march_rays_inference)
REF_ENTRY(morton3d)
REF_ENTRY(morton3d_invert)
REF_ENTRY(integrate_rays)
REF_ENTRY(integrate_rays_backward)
REF_ENTRY(integrate_rays_inference)

#ifdef NGP_REF_SHJAX
#include "spherical_harmonics_encoding.h"
extern "C" int ref_spherical_harmonics_encoding_cuda_f32(cudaStream_t s, void **b, const char *o, std::size_t n) {
    return guarded([&] { shjax::spherical_harmonics_encoding_cuda_f32(s, b, o, n); });
}
#endif

extern "C" const char *ref_last_error() { return g_err; }
