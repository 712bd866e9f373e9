/* A stand-in for another ArrayFire backend library (libafcuda behind the
 * unified loader), for testing the handle interop of libafgb300.so without
 * ArrayFire installed.  It exports the af_* entry points the interop calls,
 * with ArrayFire's signatures, over its own opaque handle type; its "device
 * memory" is whatever pointers the test hands it (a fake address on the CPU,
 * a torch allocation on a GPU).  Test infrastructure only. */
#include <stdlib.h>
#include <string.h>

typedef long long dim_t;
typedef void *af_array;
typedef int af_err;
typedef int af_dtype;

enum { AF_SUCCESS = 0, AF_ERR_NO_MEM = 101, AF_ERR_ARG = 202 };

static const unsigned kMagic = 0x5eedbeefu;
typedef struct {
    unsigned magic;
    void *ptr;
    dim_t dims[4], strides[4];
    af_dtype type;
    int locked;
} StubArray;

static char *g_pool = 0;         /* af_create_handle hands out this memory */
static size_t g_pool_bytes = 0, g_pool_used = 0;
static int g_syncs = 0, g_live = 0;

static size_t esize(af_dtype t) {
    static const size_t s[] = {4, 8, 8, 16, 1, 4, 4, 1, 8, 8, 2, 2, 2, 1};
    return (t >= 0 && t <= 13) ? s[t] : 0;
}

static StubArray *get(af_array a) {
    StubArray *s = (StubArray *)a;
    return (s && s->magic == kMagic) ? s : 0;
}

/* test hooks */
af_array stub_make_array(void *ptr, const dim_t *dims, const dim_t *strides, af_dtype type) {
    StubArray *s = (StubArray *)calloc(1, sizeof(StubArray));
    s->magic = kMagic;
    s->ptr = ptr;
    for (int i = 0; i < 4; ++i) {
        s->dims[i] = dims[i];
        s->strides[i] = strides[i];
    }
    s->type = type;
    ++g_live;
    return s;
}
void stub_set_pool(void *ptr, size_t bytes) {
    g_pool = (char *)ptr;
    g_pool_bytes = bytes;
    g_pool_used = 0;
}
int stub_is_locked(af_array a) { return get(a) ? get(a)->locked : -1; }
int stub_sync_count(void) { return g_syncs; }
int stub_live_count(void) { return g_live; }
void *stub_data(af_array a) { return get(a) ? get(a)->ptr : 0; }

/* the ArrayFire entry points (include/af/device.h, array.h, internal.h) */
af_err af_get_device_ptr(void **ptr, const af_array arr) {
    StubArray *s = get(arr);
    if (!s || !ptr) return AF_ERR_ARG;
    s->locked = 1;
    *ptr = s->ptr;
    return AF_SUCCESS;
}
af_err af_unlock_array(const af_array arr) {
    StubArray *s = get(arr);
    if (!s) return AF_ERR_ARG;
    s->locked = 0;
    return AF_SUCCESS;
}
af_err af_get_dims(dim_t *d0, dim_t *d1, dim_t *d2, dim_t *d3, const af_array arr) {
    StubArray *s = get(arr);
    if (!s) return AF_ERR_ARG;
    *d0 = s->dims[0];
    *d1 = s->dims[1];
    *d2 = s->dims[2];
    *d3 = s->dims[3];
    return AF_SUCCESS;
}
af_err af_get_strides(dim_t *s0, dim_t *s1, dim_t *s2, dim_t *s3, const af_array arr) {
    StubArray *s = get(arr);
    if (!s) return AF_ERR_ARG;
    *s0 = s->strides[0];
    *s1 = s->strides[1];
    *s2 = s->strides[2];
    *s3 = s->strides[3];
    return AF_SUCCESS;
}
af_err af_get_type(af_dtype *type, const af_array arr) {
    StubArray *s = get(arr);
    if (!s) return AF_ERR_ARG;
    *type = s->type;
    return AF_SUCCESS;
}
af_err af_sync(const int device) {
    (void)device;
    ++g_syncs;
    return AF_SUCCESS;
}
af_err af_create_handle(af_array *arr, const unsigned ndims, const dim_t *const dims,
                        const af_dtype type) {
    dim_t d[4] = {1, 1, 1, 1}, st[4];
    size_t n = 1;
    if (!arr || ndims > 4 || !esize(type)) return AF_ERR_ARG;
    for (unsigned i = 0; i < ndims; ++i) d[i] = dims[i];
    st[0] = 1;
    for (int i = 1; i < 4; ++i) st[i] = st[i - 1] * d[i - 1];
    for (int i = 0; i < 4; ++i) n *= (size_t)d[i];
    n *= esize(type);
    n = (n + 255) / 256 * 256;
    if (!g_pool || g_pool_used + n > g_pool_bytes) return AF_ERR_NO_MEM;
    *arr = stub_make_array(g_pool + g_pool_used, d, st, type);
    g_pool_used += n;
    return AF_SUCCESS;
}
af_err af_release_array(af_array arr) {
    StubArray *s = get(arr);
    if (!s) return AF_ERR_ARG;
    s->magic = 0;
    free(s);
    --g_live;
    return AF_SUCCESS;
}
