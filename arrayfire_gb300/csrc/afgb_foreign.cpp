// Interop with another ArrayFire backend library loaded in the same process.
//
// ArrayFire's af_array is an opaque pointer owned by the backend library that
// made it (src/api/c/handle.hpp:50-83); the unified loader forwards handles
// unchanged to whichever backend is active (src/api/unified/
// symbol_manager.hpp:144-165).  A binding that sends a convolution of such an
// array to this library must therefore read the array through the owning
// library's own entry points, never by dereferencing the handle.  These two
// calls do that with dlsym on the owning library's dlopen handle:
//
//   afgb_import_foreign_array: af_get_device_ptr (src/api/c/memory.cpp:121,
//     which makes the array linear on the device and locks its buffer),
//     af_get_dims, af_get_strides, af_get_type and af_sync -> a non-owning
//     view here;
//   afgb_export_foreign_array: af_create_handle + af_get_device_ptr of the
//     owning library, a device-to-device copy, then its af_unlock_array.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cstring>
#include <string>

#include "afgb_internal.hpp"
#include "conv_direct.hpp"

namespace afgb {
namespace {

typedef af_err (*GetDevicePtrFn)(void **, const af_array);
typedef af_err (*GetDimsFn)(dim_t *, dim_t *, dim_t *, dim_t *, const af_array);
typedef af_err (*GetStridesFn)(dim_t *, dim_t *, dim_t *, dim_t *, const af_array);
typedef af_err (*GetTypeFn)(af_dtype *, const af_array);
typedef af_err (*CreateHandleFn)(af_array *, const unsigned, const dim_t *const, const af_dtype);
typedef af_err (*UnlockFn)(const af_array);
typedef af_err (*ReleaseFn)(const af_array);

template <typename F>
F foreign_sym(void *lib, const char *name, bool required = true) {
    dlerror();
    void *p = dlsym(lib, name);
    if (!p && required)
        AFGB_THROW(AF_ERR_LOAD_SYM, std::string("the ArrayFire library does not export ") + name);
    return reinterpret_cast<F>(p);
}

void foreign_check(af_err e, const char *what) {
    if (e != AF_SUCCESS)
        AFGB_THROW(e, std::string("the ArrayFire library's ") + what + " failed (" +
                          std::to_string((int)e) + ")");
}

}  // namespace
}  // namespace afgb

using namespace afgb;

extern "C" af_err afgb_import_foreign_array(af_array *out, const af_array foreign,
                                            void *foreign_lib) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    AFGB_ARG_ASSERT(1, foreign != nullptr);
    AFGB_ARG_ASSERT(2, foreign_lib != nullptr);
    auto get_ptr = foreign_sym<GetDevicePtrFn>(foreign_lib, "af_get_device_ptr");
    auto get_dims = foreign_sym<GetDimsFn>(foreign_lib, "af_get_dims");
    auto get_strides = foreign_sym<GetStridesFn>(foreign_lib, "af_get_strides");
    auto get_type = foreign_sym<GetTypeFn>(foreign_lib, "af_get_type");
    // the pointer first: ArrayFire may make the array linear on this call,
    // and the strides read afterwards describe the memory it returns
    void *ptr = nullptr;
    foreign_check(get_ptr(&ptr, foreign), "af_get_device_ptr");
    dim_t d[4], s[4];
    foreign_check(get_dims(&d[0], &d[1], &d[2], &d[3], foreign), "af_get_dims");
    foreign_check(get_strides(&s[0], &s[1], &s[2], &s[3], foreign), "af_get_strides");
    af_dtype t;
    foreign_check(get_type(&t, foreign), "af_get_type");
    // the owning library's queued work on the array completes before this
    // library's stream reads it (ArrayFire's af_sync waits for its queue)
    typedef af_err (*SyncFn)(const int);
    if (auto sync = foreign_sym<SyncFn>(foreign_lib, "af_sync", false)) foreign_check(sync(-1), "af_sync");
    return afgb_device_array_view(out, ptr, 4, d, s, t);
    AFGB_CATCHALL
}

extern "C" af_err afgb_export_foreign_array(af_array *foreign_out, const af_array arr,
                                            void *foreign_lib) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, foreign_out != nullptr);
    AFGB_ARG_ASSERT(2, foreign_lib != nullptr);
    Array *a = get_array(arr);
    auto create = foreign_sym<CreateHandleFn>(foreign_lib, "af_create_handle");
    auto get_ptr = foreign_sym<GetDevicePtrFn>(foreign_lib, "af_get_device_ptr");
    auto release = foreign_sym<ReleaseFn>(foreign_lib, "af_release_array");
    auto unlock = foreign_sym<UnlockFn>(foreign_lib, "af_unlock_array", false);
    af_array h = nullptr;
    foreign_check(create(&h, 4, a->dims, a->type), "af_create_handle");
    try {
        void *dst = nullptr;
        foreign_check(get_ptr(&dst, h), "af_get_device_ptr");
        const size_t bytes = (size_t)a->elements() * dtype_size(a->type);
        if (bytes) {
            const Array src = a->is_linear() ? *a : make_dense(*a);
            // the owning library runs on its own stream: the copy is made
            // and waited for here, so its next call sees the data
            AFGB_CUDA(cudaMemcpyAsync(dst, src.data(), bytes, cudaMemcpyDeviceToDevice, stream()));
            AFGB_CUDA(cudaStreamSynchronize(stream()));
        }
        if (unlock) foreign_check(unlock(h), "af_unlock_array");
    } catch (...) {
        release(h);
        throw;
    }
    *foreign_out = h;
    AFGB_CATCHALL
}
