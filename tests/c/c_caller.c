/* A plain C caller of libafgb300's ArrayFire-named entry points: the
 * convolution call sequence of the reference's documentation (create, convolve,
 * read back, release, error strings).  Compiled by tests/test_c_abi.py; with
 * an argument "run" it exercises the library on the GPU and prints one
 * line "ok <checksum>". */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "afgb300.h"

static int check(af_err e, const char *what) {
    if (e != AF_SUCCESS) {
        char *msg = NULL;
        dim_t len = 0;
        af_get_last_error(&msg, &len);
        fprintf(stderr, "%s failed: %d (%s) %s\n", what, (int)e, af_err_to_string(e),
                msg ? msg : "");
        if (msg) af_free_host(msg);
        return 1;
    }
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2 || strcmp(argv[1], "run") != 0) {
        /* link check only: the error table needs no device */
        printf("%s\n", af_err_to_string(AF_ERR_ARG));
        return 0;
    }
    /* 3x3 image of 1..9 convolved with a 3x3 box of ones, DEFAULT mode: each
     * output is the sum of the in-range 3x3 neighbourhood */
    float img[9], box[9], out[9];
    for (int i = 0; i < 9; ++i) {
        img[i] = (float)(i + 1);
        box[i] = 1.0f;
    }
    dim_t d[2] = {3, 3};
    af_array s = 0, f = 0, o = 0;
    if (check(af_create_array(&s, img, 2, d, f32), "af_create_array")) return 1;
    if (check(af_create_array(&f, box, 2, d, f32), "af_create_array")) return 1;
    if (check(af_convolve2(&o, s, f, AF_CONV_DEFAULT, AF_CONV_SPATIAL), "af_convolve2")) return 1;
    dim_t n = 0;
    if (check(af_get_elements(&n, o), "af_get_elements") || n != 9) return 1;
    if (check(af_get_data_ptr(out, o), "af_get_data_ptr")) return 1;
    const float expect[9] = {12, 21, 16, 27, 45, 33, 24, 39, 28};
    double sum = 0;
    for (int i = 0; i < 9; ++i) {
        if (out[i] != expect[i]) {
            fprintf(stderr, "out[%d] = %g, expected %g\n", i, out[i], expect[i]);
            return 1;
        }
        sum += out[i];
    }
    /* a reference error code: three stride dims for the NN call (ARG,
     * src/api/c/convolve.cpp:365) */
    af_array bad = 0;
    dim_t st[3] = {1, 1, 2}, pd[2] = {0, 0}, dl[2] = {1, 1};
    af_err e = af_convolve2_nn(&bad, s, f, 3, st, 2, pd, 2, dl);
    if (e != AF_ERR_ARG) {
        fprintf(stderr, "af_convolve2_nn with 3 stride dims returned %d\n", (int)e);
        return 1;
    }
    af_release_array(o);
    af_release_array(f);
    af_release_array(s);
    printf("ok %.0f\n", sum);
    return 0;
}
