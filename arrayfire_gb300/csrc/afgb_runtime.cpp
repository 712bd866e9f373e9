// Runtime of libafgb300: error state, device memory, streams and the array
// lifecycle exports (the af_array subset of include/af/array.h and
// include/af/device.h that the convolution path needs).
//
// Design: one process, one GPU at a time.  Device memory comes from the
// CUDA stream-ordered pool (cudaMallocAsync) with its release threshold
// raised, so freed blocks stay cached for the next call — the role of the
// reference's DefaultMemoryManager (src/backend/common/DefaultMemoryManager.cpp)
// without its bookkeeping.  Work runs on one non-blocking stream per device,
// or on a stream the caller installs (afgb_set_stream).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "afgb_internal.hpp"

namespace afgb {

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;

static bool print_errors() {
    static int v = [] {
        const char *e = std::getenv("AF_PRINT_ERRORS");
        return (e && e[0] && e[0] != '0') ? 1 : 0;
    }();
    return v != 0;
}

[[noreturn]] void throw_err(af_err code, const char *file, int line, const std::string &msg) {
    std::string full = msg + "\nIn " + file + ":" + std::to_string(line);
    throw AfError(code, full);
}

void cuda_check(cudaError_t e, const char *what, const char *file, int line) {
    if (e == cudaSuccess) return;
    af_err code = (e == cudaErrorMemoryAllocation) ? AF_ERR_NO_MEM : AF_ERR_RUNTIME;
    throw_err(code, file, line, std::string("CUDA error ") + cudaGetErrorName(e) + " (" +
                                    cudaGetErrorString(e) + ") in " + what);
}

static bool synchronous_calls() {
    // AF_SYNCHRONOUS_CALLS (src/backend/cuda/debug_cuda.hpp:64-72)
    static int v = [] {
        const char *e = std::getenv("AF_SYNCHRONOUS_CALLS");
        return (e && e[0] == '1') ? 1 : 0;
    }();
    return v != 0;
}

void post_launch(const char *kernel_name) {
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw_err(AF_ERR_RUNTIME, __FILE__, __LINE__,
                  std::string("kernel launch failed: ") + kernel_name + ": " +
                      cudaGetErrorString(e));
    }
    if (synchronous_calls()) AFGB_CUDA(cudaStreamSynchronize(stream()));
}

af_err record_exception() {
    af_err code = AF_ERR_UNKNOWN;
    try {
        throw;
    } catch (const AfError &e) {
        code = e.code;
        g_last_error = e.what();
    } catch (const std::bad_alloc &e) {
        code = AF_ERR_NO_MEM;
        g_last_error = std::string("host allocation failed: ") + e.what();
    } catch (const std::exception &e) {
        code = AF_ERR_INTERNAL;
        g_last_error = e.what();
    } catch (...) {
        code = AF_ERR_UNKNOWN;
        g_last_error = "unknown error";
    }
    if (print_errors()) std::fprintf(stderr, "[afgb300] %s\n", g_last_error.c_str());
    return code;
}

// ---------------------------------------------------------------- dtypes
size_t dtype_size(af_dtype t) {
    switch (t) {
        case f32: return 4;
        case c32: return 8;
        case f64: return 8;
        case c64: return 16;
        case b8: return 1;
        case s32: return 4;
        case u32: return 4;
        case u8: return 1;
        case s64: return 8;
        case u64: return 8;
        case s16: return 2;
        case u16: return 2;
        case f16: return 2;
        case s8: return 1;
    }
    return 0;
}
bool dtype_valid(af_dtype t) { return (int)t >= 0 && (int)t <= (int)s8; }

// ---------------------------------------------------------------- state
namespace {
struct DevState {
    cudaStream_t own = nullptr;
    cudaStream_t h2d = nullptr;  // af_create_array uploads
    cudaStream_t d2h = nullptr;  // af_get_data_ptr downloads
    bool pool_ready = false;
    int sms = 0;
};
std::mutex g_mu;
DevState g_dev[64];
cudaStream_t g_user_stream = nullptr;
bool g_user_stream_set = false;
std::atomic<int> g_exact{0};
std::atomic<int> g_fail_after{0};
std::atomic<unsigned long long> g_launches{0};
}  // namespace

int device() {
    int d = 0;
    AFGB_CUDA(cudaGetDevice(&d));
    if (d < 0 || d >= 64) AFGB_THROW(AF_ERR_DEVICE, "device ordinal out of range");
    return d;
}

static DevState &dev_state(int d) {
    DevState &s = g_dev[d];
    if (!s.pool_ready) {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!s.pool_ready) {
            AFGB_CUDA(cudaStreamCreateWithFlags(&s.own, cudaStreamNonBlocking));
            AFGB_CUDA(cudaStreamCreateWithFlags(&s.h2d, cudaStreamNonBlocking));
            AFGB_CUDA(cudaStreamCreateWithFlags(&s.d2h, cudaStreamNonBlocking));
            cudaMemPool_t pool;
            AFGB_CUDA(cudaDeviceGetDefaultMemPool(&pool, d));
            uint64_t thr = UINT64_MAX;
            AFGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
            AFGB_CUDA(cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, d));
            s.pool_ready = true;
        }
    }
    return s;
}

cudaStream_t stream() {
    if (g_user_stream_set) return g_user_stream;
    return dev_state(device()).own;
}

int num_sms() { return dev_state(device()).sms; }

unsigned int tma_take_error();
void tma_set_wait_limit(unsigned int polls, int skip_block0);
void tc_set_wait_limit(unsigned int polls);

void check_device_errors() {
    unsigned int w = tc_take_error() | tma_take_error();
    if (w) {
        AFGB_THROW(AF_ERR_RUNTIME, "a tensor-core kernel pipeline wait timed out (code " +
                                       std::to_string(w) + "); its results are invalid");
    }
}
namespace {
thread_local int t_exact_depth = 0;
}
bool exact_fp() { return t_exact_depth > 0 || g_exact.load() != 0; }
ExactScope::ExactScope() { ++t_exact_depth; }
ExactScope::~ExactScope() { --t_exact_depth; }
void count_launch(unsigned n) { g_launches += n; }

// ---------------------------------------------------------------- memory
// Every pool allocation is recorded with its size and the purpose tag that
// was current on the allocating thread (MemTag), so that af_device_mem_info
// can report the bytes and buffers in use, and afgb_device_mem_peak the peak
// since the last reset together with the bytes each purpose held at it.
namespace {
thread_local const char *t_mem_tag = "scratch";
struct LiveBuf {
    size_t bytes;
    const char *tag;
};
struct MemBook {
    std::mutex mu;
    std::unordered_map<void *, LiveBuf> live;
    std::map<std::string, size_t> by_tag, peak_by_tag;
    size_t bytes = 0, peak = 0;
};
MemBook &mem_book() {
    static MemBook *b = new MemBook();  // outlives static destructors of callers
    return *b;
}
void book_alloc(void *p, size_t bytes) {
    MemBook &b = mem_book();
    std::lock_guard<std::mutex> lk(b.mu);
    b.live[p] = LiveBuf{bytes, t_mem_tag};
    b.bytes += bytes;
    b.by_tag[t_mem_tag] += bytes;
    if (b.bytes > b.peak) {
        b.peak = b.bytes;
        b.peak_by_tag = b.by_tag;
    }
}
void book_free(void *p) {
    MemBook &b = mem_book();
    std::lock_guard<std::mutex> lk(b.mu);
    auto it = b.live.find(p);
    if (it == b.live.end()) return;
    b.bytes -= it->second.bytes;
    b.by_tag[it->second.tag] -= it->second.bytes;
    b.live.erase(it);
}
}  // namespace

MemTag::MemTag(const char *tag) : prev(t_mem_tag) { t_mem_tag = tag; }
MemTag::~MemTag() { t_mem_tag = prev; }

void *alloc_device(size_t bytes) {
    int fa = g_fail_after.load();
    if (fa > 0) {
        if (g_fail_after.fetch_sub(1) == 1) {
            AFGB_THROW(AF_ERR_NO_MEM, "device allocation failed (injected)");
        }
    }
    if (bytes == 0) bytes = 16;
    void *p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, bytes, stream());
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        AFGB_THROW(AF_ERR_NO_MEM, "device allocation of " + std::to_string(bytes) +
                                      " bytes failed: " + cudaGetErrorString(e));
    }
    book_alloc(p, bytes);
    return p;
}

void free_device(void *p) {
    if (!p) return;
    book_free(p);
    (void)cudaFreeAsync(p, stream());
}

static cudaEvent_t new_event() {
    cudaEvent_t e = nullptr;
    AFGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return e;
}

void Buffer::drop_derived() {
    std::lock_guard<std::mutex> lk(derived_mu);
    if (derived) free_device(derived);
    derived = nullptr;
    derived_key = 0;
    derived_stream = nullptr;
}

Buffer::~Buffer() {
    if (derived) free_device(derived);
    if (ptr && upload_pending.load()) (void)cudaStreamWaitEvent(stream(), uploaded, 0);
    if (uploaded) (void)cudaEventDestroy(uploaded);
    if (written) (void)cudaEventDestroy(written);
    if (!ptr) return;
    if (kind == BufKind::Pool) {
        free_device(ptr);
    } else if (kind == BufKind::Adopted) {
        (void)cudaFree(ptr);
    }
}

// ---------------------------------------------------------------- arrays
dim_t dim4_ndims(const dim_t d[4]) {
    dim_t num = d[0] * d[1] * d[2] * d[3];
    if (num == 0) return 0;
    if (num == 1) return 1;
    if (d[3] != 1) return 4;
    if (d[2] != 1) return 3;
    if (d[1] != 1) return 2;
    return 1;
}

void dim4_from(dim_t out[4], unsigned n, const dim_t *vals) {
    for (unsigned i = 0; i < 4; ++i) out[i] = (n > i) ? vals[i] : 1;
}

dim_t Array::ndims() const { return dim4_ndims(dims); }

bool Array::is_linear() const {
    dim_t s = 1;
    for (int i = 0; i < 4; ++i) {
        if (dims[i] != 1 && strides[i] != s) return false;
        s *= dims[i];
    }
    return true;
}

static void dense_strides(Array *a) {
    a->strides[0] = 1;
    for (int i = 1; i < 4; ++i) a->strides[i] = a->strides[i - 1] * a->dims[i - 1];
}

static const uint64_t kMagic = 0xAF6B300A11A5ull;
struct Handle {
    uint64_t magic = kMagic;
    Array arr;
};

Array *get_array(const af_array a) {
    if (!a) AFGB_THROW(AF_ERR_ARG, "Invalid (null) af_array handle");
    Handle *h = static_cast<Handle *>(a);
    if (h->magic != kMagic) AFGB_THROW(AF_ERR_ARG, "Invalid af_array handle");
    Buffer *b = h->arr.buf.get();
    if (b && b->upload_pending.exchange(false))
        AFGB_CUDA(cudaStreamWaitEvent(stream(), b->uploaded, 0));  // its upload first
    return &h->arr;
}

void mark_written(const Array &a) {
    Buffer *b = a.buf.get();
    if (!b || b->kind != BufKind::Pool) return;
    if (b->derived) b->drop_derived();  // new contents: the derived copy is stale
    if (!b->written) b->written = new_event();
    AFGB_CUDA(cudaEventRecord(b->written, stream()));
}

af_array make_handle(Array *a) {
    Handle *h = new Handle();
    h->arr = *a;
    mark_written(*a);  // every operation hands its outputs out through here
    return static_cast<af_array>(h);
}

Array *create_array(af_dtype t, const dim_t dims[4]) {
    static thread_local Array scratch;
    scratch = Array();
    scratch.type = t;
    for (int i = 0; i < 4; ++i) {
        if (dims[i] < 0) AFGB_THROW(AF_ERR_SIZE, "negative dimension");
        scratch.dims[i] = dims[i];
    }
    dense_strides(&scratch);
    auto b = std::make_shared<Buffer>();
    b->bytes = (size_t)scratch.elements() * dtype_size(t);
    {
        MemTag tag("arrays");
        b->ptr = alloc_device(b->bytes);
    }
    b->kind = BufKind::Pool;
    b->device = device();
    scratch.buf = b;
    return &scratch;
}

// ---------------------------------------------------------------- timing
namespace {
struct TimedLaunch {
    std::string name;
    cudaEvent_t a, b;
};
std::mutex g_tmu;
std::atomic<int> g_timing{0};
std::vector<TimedLaunch> g_timed;
}  // namespace

KernelTimer::KernelTimer(const char *n) : name(n) {
    if (!g_timing.load()) return;
    if (cudaEventCreate(&start) != cudaSuccess) {
        start = nullptr;
        return;
    }
    cudaEventRecord(start, stream());
}

KernelTimer::~KernelTimer() {
    if (!start) return;
    cudaEvent_t end;
    if (cudaEventCreate(&end) != cudaSuccess) {
        cudaEventDestroy(start);
        return;
    }
    cudaEventRecord(end, stream());
    std::lock_guard<std::mutex> lk(g_tmu);
    g_timed.push_back(TimedLaunch{name, start, end});
}

}  // namespace afgb

using namespace afgb;

// ======================================================================
// exported lifecycle API
// ======================================================================
extern "C" {

af_err af_create_handle(af_array *arr, const unsigned ndims, const dim_t *const dims,
                        const af_dtype type) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, arr != nullptr);
    if (!dtype_valid(type)) AFGB_TYPE_ERROR(4, type);
    AFGB_ARG_ASSERT(1, ndims <= 4);
    dim_t d[4];
    dim4_from(d, ndims, dims);
    *arr = make_handle(create_array(type, d));
    AFGB_CATCHALL
}

af_err af_create_array(af_array *arr, const void *const data, const unsigned ndims,
                       const dim_t *const dims, const af_dtype type) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, arr != nullptr);
    if (!dtype_valid(type)) AFGB_TYPE_ERROR(4, type);
    AFGB_ARG_ASSERT(2, ndims <= 4);
    dim_t d[4];
    dim4_from(d, ndims, dims);
    Array *a = create_array(type, d);
    size_t bytes = (size_t)a->elements() * dtype_size(type);
    if (bytes && data) {
        // upload on the copy stream, after the stream-ordered allocation; the
        // compute stream waits for it at the array's first use (get_array).
        // As in ArrayFire (src/backend/cuda/Array.cpp:107-111) the call
        // returns once the host buffer has been read, so the caller may reuse
        // it; work already queued on the compute stream keeps running meanwhile
        DevState &ds = dev_state(device());
        cudaEvent_t allocated = new_event();
        AFGB_CUDA(cudaEventRecord(allocated, stream()));
        AFGB_CUDA(cudaStreamWaitEvent(ds.h2d, allocated, 0));
        (void)cudaEventDestroy(allocated);
        AFGB_CUDA(cudaMemcpyAsync(a->data(), data, bytes, cudaMemcpyHostToDevice, ds.h2d));
        Buffer *b = a->buf.get();
        b->uploaded = new_event();
        AFGB_CUDA(cudaEventRecord(b->uploaded, ds.h2d));
        b->upload_pending.store(true);
        AFGB_CUDA(cudaEventSynchronize(b->uploaded));
    }
    *arr = make_handle(a);
    AFGB_CATCHALL
}

af_err af_device_array(af_array *arr, void *data, const unsigned ndims,
                       const dim_t *const dims, const af_dtype type) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, arr != nullptr);
    if (!dtype_valid(type)) AFGB_TYPE_ERROR(4, type);
    AFGB_ARG_ASSERT(2, ndims <= 4);
    Array a;
    a.type = type;
    dim4_from(a.dims, ndims, dims);
    dense_strides(&a);
    auto b = std::make_shared<Buffer>();
    b->ptr = data;
    b->bytes = (size_t)a.elements() * dtype_size(type);
    b->kind = BufKind::Adopted;
    b->device = device();
    a.buf = b;
    *arr = make_handle(&a);
    AFGB_CATCHALL
}

af_err afgb_device_array_view(af_array *arr, void *data, const unsigned ndims,
                              const dim_t *const dims, const dim_t *const strides,
                              const af_dtype type) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, arr != nullptr);
    if (!dtype_valid(type)) AFGB_TYPE_ERROR(5, type);
    AFGB_ARG_ASSERT(2, ndims <= 4);
    Array a;
    a.type = type;
    dim4_from(a.dims, ndims, dims);
    if (strides) {
        for (unsigned i = 0; i < 4; ++i) {
            a.strides[i] = (i < ndims) ? strides[i] : (i == 0 ? 1 : a.strides[i - 1] * a.dims[i - 1]);
        }
    } else {
        dense_strides(&a);
    }
    auto b = std::make_shared<Buffer>();
    b->ptr = data;
    b->kind = BufKind::View;
    // a view reads and writes nothing here; without a usable device (host-side
    // binding tests) it is recorded against device 0
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        dev = 0;
    }
    b->device = dev;
    a.buf = b;
    *arr = make_handle(&a);
    AFGB_CATCHALL
}

af_err af_get_data_ptr(void *data, const af_array arr) {
    AFGB_TRY
    Array *a = get_array(arr);
    AFGB_ARG_ASSERT(0, data != nullptr);
    size_t es = dtype_size(a->type);
    if (a->elements() == 0) return AF_SUCCESS;
    Buffer *b = a->buf.get();
    if (a->is_linear() && b && b->kind == BufKind::Pool && b->written) {
        // on the download stream, after the last write only: the copy
        // overlaps whatever the compute stream has queued since
        DevState &ds = dev_state(device());
        AFGB_CUDA(cudaStreamWaitEvent(ds.d2h, b->written, 0));
        if (b->uploaded) AFGB_CUDA(cudaStreamWaitEvent(ds.d2h, b->uploaded, 0));
        AFGB_CUDA(cudaMemcpyAsync(data, a->data(), (size_t)a->elements() * es,
                                  cudaMemcpyDeviceToHost, ds.d2h));
        AFGB_CUDA(cudaStreamSynchronize(ds.d2h));
        check_device_errors();
        return AF_SUCCESS;
    }
    if (a->is_linear()) {
        AFGB_CUDA(cudaMemcpyAsync(data, a->data(), (size_t)a->elements() * es,
                                  cudaMemcpyDeviceToHost, stream()));
    } else {
        // strided view: one 2-D copy per (d2, d3) slice row set
        char *dst = static_cast<char *>(data);
        for (dim_t k3 = 0; k3 < a->dims[3]; ++k3)
            for (dim_t k2 = 0; k2 < a->dims[2]; ++k2)
                for (dim_t k1 = 0; k1 < a->dims[1]; ++k1) {
                    const char *src = static_cast<const char *>(a->data()) +
                                      (k1 * a->strides[1] + k2 * a->strides[2] +
                                       k3 * a->strides[3]) * (dim_t)es;
                    AFGB_CUDA(cudaMemcpy2DAsync(dst, es, src, a->strides[0] * es, es,
                                                (size_t)a->dims[0], cudaMemcpyDeviceToHost,
                                                stream()));
                    dst += a->dims[0] * es;
                }
    }
    AFGB_CUDA(cudaStreamSynchronize(stream()));
    check_device_errors();
    AFGB_CATCHALL
}

af_err af_get_device_ptr(void **ptr, const af_array arr) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, ptr != nullptr);
    Array *a = get_array(arr);
    // the caller may now write through the pointer on a stream of its own:
    // later downloads of this buffer go back to waiting on the whole stream
    if (Buffer *b = a->buf.get()) {
        if (b->written) (void)cudaEventDestroy(b->written);
        b->written = nullptr;
        b->drop_derived();  // nor can a copy derived from its contents be kept
    }
    *ptr = a->data();
    AFGB_CATCHALL
}

af_err af_release_array(af_array arr) {
    AFGB_TRY
    if (!arr) return AF_SUCCESS;
    get_array(arr);
    Handle *h = static_cast<Handle *>(arr);
    h->magic = 0;
    delete h;
    AFGB_CATCHALL
}

af_err af_retain_array(af_array *out, const af_array in) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    *out = make_handle(get_array(in));
    AFGB_CATCHALL
}

af_err af_get_elements(dim_t *elems, const af_array arr) {
    AFGB_TRY
    *elems = get_array(arr)->elements();
    AFGB_CATCHALL
}

af_err af_get_type(af_dtype *type, const af_array arr) {
    AFGB_TRY
    *type = get_array(arr)->type;
    AFGB_CATCHALL
}

af_err af_get_dims(dim_t *d0, dim_t *d1, dim_t *d2, dim_t *d3, const af_array arr) {
    AFGB_TRY
    Array *a = get_array(arr);
    *d0 = a->dims[0];
    *d1 = a->dims[1];
    *d2 = a->dims[2];
    *d3 = a->dims[3];
    AFGB_CATCHALL
}

af_err af_get_numdims(unsigned *result, const af_array arr) {
    AFGB_TRY
    *result = (unsigned)get_array(arr)->ndims();
    AFGB_CATCHALL
}

af_err af_get_strides(dim_t *s0, dim_t *s1, dim_t *s2, dim_t *s3, const af_array arr) {
    AFGB_TRY
    Array *a = get_array(arr);
    *s0 = a->strides[0];
    *s1 = a->strides[1];
    *s2 = a->strides[2];
    *s3 = a->strides[3];
    AFGB_CATCHALL
}

static void sync_current_device() {
    DevState &ds = dev_state(device());
    AFGB_CUDA(cudaStreamSynchronize(ds.h2d));
    AFGB_CUDA(cudaStreamSynchronize(stream()));
    AFGB_CUDA(cudaStreamSynchronize(ds.d2h));
    check_device_errors();
}

af_err af_sync(const int dev) {
    AFGB_TRY
    if (dev >= 0) {
        int cur = device();
        if (dev != cur) AFGB_CUDA(cudaSetDevice(dev));
        sync_current_device();
        if (dev != cur) AFGB_CUDA(cudaSetDevice(cur));
    } else {
        sync_current_device();
    }
    AFGB_CATCHALL
}

af_err af_device_mem_info(size_t *alloc_bytes, size_t *alloc_buffers, size_t *lock_bytes,
                          size_t *lock_buffers) {
    AFGB_TRY
    MemBook &b = mem_book();
    size_t live_bytes, live_bufs;
    {
        std::lock_guard<std::mutex> lk(b.mu);
        live_bytes = b.bytes;
        live_bufs = b.live.size();
    }
    uint64_t reserved = live_bytes;
    cudaMemPool_t pool;
    int d = device();
    (void)dev_state(d);
    if (cudaDeviceGetDefaultMemPool(&pool, d) == cudaSuccess) {
        uint64_t r = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r) == cudaSuccess)
            reserved = r;
    }
    (void)cudaGetLastError();
    if (alloc_bytes) *alloc_bytes = (size_t)reserved;
    if (alloc_buffers) *alloc_buffers = live_bufs;
    if (lock_bytes) *lock_bytes = live_bytes;
    if (lock_buffers) *lock_buffers = live_bufs;
    AFGB_CATCHALL
}

af_err af_device_gc() {
    AFGB_TRY
    int d = device();
    (void)dev_state(d);
    AFGB_CUDA(cudaStreamSynchronize(stream()));
    cudaMemPool_t pool;
    AFGB_CUDA(cudaDeviceGetDefaultMemPool(&pool, d));
    AFGB_CUDA(cudaMemPoolTrimTo(pool, 0));
    AFGB_CATCHALL
}

af_err afgb_device_mem_peak(size_t *peak_bytes, int reset) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, peak_bytes != nullptr);
    MemBook &b = mem_book();
    std::lock_guard<std::mutex> lk(b.mu);
    *peak_bytes = b.peak;
    if (reset) {
        b.peak = b.bytes;
        b.peak_by_tag = b.by_tag;
    }
    AFGB_CATCHALL
}

af_err afgb_device_mem_peak_breakdown(char *buf, size_t len) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, buf != nullptr && len > 0);
    std::string out;
    {
        MemBook &b = mem_book();
        std::lock_guard<std::mutex> lk(b.mu);
        for (const auto &kv : b.peak_by_tag)
            if (kv.second) out += kv.first + "=" + std::to_string(kv.second) + "\n";
    }
    const size_t n = std::min(len - 1, out.size());
    std::memcpy(buf, out.data(), n);
    buf[n] = 0;
    AFGB_CATCHALL
}

af_err af_free_host(void *ptr) {
    std::free(ptr);
    return AF_SUCCESS;
}

void af_get_last_error(char **msg, dim_t *len) {
    if (!msg) return;
    const std::string &s = g_last_error;
    char *m = static_cast<char *>(std::malloc(s.size() + 1));
    if (!m) {
        *msg = nullptr;
        if (len) *len = 0;
        return;
    }
    std::memcpy(m, s.c_str(), s.size() + 1);
    *msg = m;
    if (len) *len = (dim_t)s.size();
    g_last_error.clear();
}

const char *af_err_to_string(const af_err err) {
    switch (err) {
        case AF_SUCCESS: return "Success";
        case AF_ERR_NO_MEM: return "Device out of memory";
        case AF_ERR_DRIVER: return "Driver not available or incompatible";
        case AF_ERR_RUNTIME: return "Runtime error ";
        case AF_ERR_INVALID_ARRAY: return "Invalid array";
        case AF_ERR_ARG: return "Invalid input argument";
        case AF_ERR_SIZE: return "Invalid input size";
        case AF_ERR_TYPE: return "Function does not support this data type";
        case AF_ERR_DIFF_TYPE: return "Input types are not the same";
        case AF_ERR_BATCH: return "Invalid batch configuration";
        case AF_ERR_DEVICE: return "Input does not belong to the current device.";
        case AF_ERR_NOT_SUPPORTED: return "Function not supported";
        case AF_ERR_NOT_CONFIGURED: return "Function not configured to build";
        case AF_ERR_NONFREE: return "Function unavailable. ArrayFire compiled without Non-Free algorithms support";
        case AF_ERR_NO_DBL: return "Double precision not supported for this device";
        case AF_ERR_NO_GFX: return "Graphics functionality unavailable. ArrayFire compiled without Graphics support";
        case AF_ERR_NO_HALF: return "Half precision floats not supported for this device";
        case AF_ERR_LOAD_LIB: return "Failed to load dynamic library. ";
        case AF_ERR_LOAD_SYM: return "Failed to load symbol";
        case AF_ERR_ARR_BKND_MISMATCH: return "There was a mismatch between an array and the current backend";
        case AF_ERR_INTERNAL: return "Internal error";
        case AF_ERR_UNKNOWN: return "Unknown error";
    }
    return "Unknown error. Please open an issue and add this error code to the case in af_err_to_string.";
}

af_err afgb_set_stream(void *s) {
    AFGB_TRY
    g_user_stream = static_cast<cudaStream_t>(s);
    g_user_stream_set = (s != nullptr);
    AFGB_CATCHALL
}

af_err afgb_get_stream(void **s) {
    AFGB_TRY
    *s = static_cast<void *>(stream());
    AFGB_CATCHALL
}

af_err afgb_set_exact_fp(int exact) {
    g_exact.store(exact ? 1 : 0);
    return AF_SUCCESS;
}

void afgb_debug_fail_alloc_after(int n) { g_fail_after.store(n > 0 ? n : 0); }

af_err afgb_debug_wait_limit(unsigned int polls, int skip_first_block_copies) {
    AFGB_TRY
    tma_set_wait_limit(polls, skip_first_block_copies ? 1 : 0);
    tc_set_wait_limit(polls);
    AFGB_CATCHALL
}

unsigned long long afgb_kernel_launch_count(void) { return g_launches.load(); }

void afgb_kernel_timing(int enable) {
    g_timing.store(enable ? 1 : 0);
    if (!enable) {
        std::lock_guard<std::mutex> lk(g_tmu);
        for (auto &t : g_timed) {
            cudaEventDestroy(t.a);
            cudaEventDestroy(t.b);
        }
        g_timed.clear();
    }
}

af_err afgb_kernel_time(const char *name, unsigned long long *count, double *total_ms) {
    AFGB_TRY
    std::lock_guard<std::mutex> lk(g_tmu);
    unsigned long long c = 0;
    double tot = 0.0;
    for (auto &t : g_timed) {
        if (name && t.name != name) continue;
        AFGB_CUDA(cudaEventSynchronize(t.b));
        float ms = 0.f;
        AFGB_CUDA(cudaEventElapsedTime(&ms, t.a, t.b));
        tot += ms;
        ++c;
    }
    if (count) *count = c;
    if (total_ms) *total_ms = tot;
    AFGB_CATCHALL
}

const char *afgb_version(void) { return "afgb300 0.1 (ArrayFire 3.10 convolution C ABI, sm_103a)"; }

}  // extern "C"
