// Internal runtime of libafgb300: the array object, error plumbing, device
// memory and stream state shared by the C-ABI layer and the kernel launchers.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include "afgb300.h"

namespace afgb {

// ---------------------------------------------------------------------------
// errors: every exported function catches these and turns them into af_err
// (the reference's CATCHALL / processException, src/backend/common/
// err_common.hpp:149-200, err_common.cpp:117-125).
// ---------------------------------------------------------------------------
struct AfError : public std::runtime_error {
    af_err code;
    AfError(af_err c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

[[noreturn]] void throw_err(af_err code, const char *file, int line, const std::string &msg);

#define AFGB_THROW(code, msg) ::afgb::throw_err((code), __FILE__, __LINE__, (msg))
// ARG_ASSERT / DIM_ASSERT / TYPE_ERROR carry the argument index like the
// reference's macros (src/backend/common/err_common.hpp).
#define AFGB_ARG_ASSERT(idx, cond)                                                     \
    do {                                                                               \
        if (!(cond)) AFGB_THROW(AF_ERR_ARG, "Invalid argument at index " #idx ": " #cond); \
    } while (0)
#define AFGB_DIM_ASSERT(idx, cond)                                                    \
    do {                                                                              \
        if (!(cond)) AFGB_THROW(AF_ERR_SIZE, "Invalid dimension at index " #idx ": " #cond); \
    } while (0)
#define AFGB_TYPE_ERROR(idx, t) \
    AFGB_THROW(AF_ERR_TYPE, "Invalid type at index " #idx ": " + std::to_string((int)(t)))

void cuda_check(cudaError_t e, const char *what, const char *file, int line);
#define AFGB_CUDA(call) ::afgb::cuda_check((call), #call, __FILE__, __LINE__)
// after every launch (POST_LAUNCH_CHECK, src/backend/cuda/debug_cuda.hpp:57-72)
void post_launch(const char *kernel_name);
#define AFGB_POST_LAUNCH(name) ::afgb::post_launch(name)

af_err record_exception();  // used inside catch(...) blocks

#define AFGB_TRY try {
#define AFGB_CATCHALL             \
    }                             \
    catch (...) {                 \
        return ::afgb::record_exception(); \
    }                             \
    return AF_SUCCESS;

// ---------------------------------------------------------------------------
// dtype traits
// ---------------------------------------------------------------------------
size_t dtype_size(af_dtype t);
bool dtype_valid(af_dtype t);

// ---------------------------------------------------------------------------
// device buffers and arrays
// ---------------------------------------------------------------------------
enum class BufKind { Pool, Adopted, View };

struct Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    BufKind kind = BufKind::Pool;
    int device = 0;
    // host transfers run on the library's copy streams so that they overlap
    // compute: `uploaded` completes the af_create_array copy (the compute
    // stream waits on it once, at the first use); `written` is recorded on the
    // compute stream after the last operation that wrote the buffer, and
    // af_get_data_ptr's copy waits on it instead of on the whole stream
    cudaEvent_t uploaded = nullptr;
    std::atomic<bool> upload_pending{false};
    cudaEvent_t written = nullptr;
    // a device copy derived from this buffer's contents (the bf16
    // channels-last operand of the tensor-core kernels), made on
    // `derived_stream` and keyed by the layout it was made for; it stays
    // valid until the buffer is written (mark_written), handed to the caller
    // for writing (af_get_device_ptr) or freed.  Pool buffers only: the
    // library sees every write to those.
    std::mutex derived_mu;
    void *derived = nullptr;
    unsigned long long derived_key = 0;
    cudaStream_t derived_stream = nullptr;
    void drop_derived();
    ~Buffer();
};

struct Array {
    af_dtype type = f32;
    dim_t dims[4] = {1, 1, 1, 1};
    dim_t strides[4] = {1, 1, 1, 1};
    dim_t offset = 0;  // elements
    std::shared_ptr<Buffer> buf;

    dim_t elements() const { return dims[0] * dims[1] * dims[2] * dims[3]; }
    // af::dim4::ndims (src/backend/common/dim4.cpp:48-58)
    dim_t ndims() const;
    bool is_linear() const;  // dense column-major
    void *data() const {
        return buf ? static_cast<char *>(buf->ptr) + offset * (dim_t)dtype_size(type) : nullptr;
    }
    template <typename T>
    T *ptr() const { return static_cast<T *>(data()); }
};

// the af::dim4 rule for a dims list (used for stride/padding/dilation too):
// dims beyond `n` are 1 (src/backend/common/dim4.cpp:35-37)
void dim4_from(dim_t out[4], unsigned n, const dim_t *vals);
dim_t dim4_ndims(const dim_t d[4]);

Array *get_array(const af_array a);       // validates the handle; orders a pending upload
// record that the compute stream has just enqueued the last write of `a`'s
// buffer (pool buffers only; af_get_data_ptr then copies after that point)
void mark_written(const Array &a);
af_array make_handle(Array *a);
// a new dense array on the current device/stream
Array *create_array(af_dtype t, const dim_t dims[4]);
// raw stream-ordered scratch (freed with free_scratch on the same stream)
void *alloc_device(size_t bytes);
void free_device(void *p);
// the purpose recorded with the allocations this thread makes while the
// object lives (reported by afgb_device_mem_peak_breakdown); `tag` must be a
// string literal
struct MemTag {
    const char *prev;
    explicit MemTag(const char *tag);
    ~MemTag();
};

// ---------------------------------------------------------------------------
// execution state
// ---------------------------------------------------------------------------
cudaStream_t stream();
// error word of the tensor-core kernels (bounded waits that timed out);
// read and cleared after the host has synchronised
unsigned int tc_take_error();
void check_device_errors();
int device();
bool exact_fp();
// while one lives, exact_fp() is true on this thread (for callers whose
// results feed discrete decisions, e.g. the corner detector's window sums,
// which must round like the reference whatever the global setting)
struct ExactScope {
    ExactScope();
    ~ExactScope();
};
int num_sms();
void count_launch(unsigned n = 1);

// Optional per-kernel device timing (afgb_kernel_timing): when enabled, the
// launchers bracket their main kernels with CUDA events on the launch stream.
struct KernelTimer {
    const char *name;
    cudaEvent_t start = nullptr;
    KernelTimer(const char *n);
    ~KernelTimer();
};

// direct-convolution batch kinds (src/backend/common/internal_enums.hpp:12-22)
enum BatchKind { BATCH_NONE = 0, BATCH_LHS, BATCH_RHS, BATCH_SAME, BATCH_DIFF, BATCH_UNSUPPORTED };

}  // namespace afgb
