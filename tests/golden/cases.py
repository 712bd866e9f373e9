"""Seeded case matrix shared by the golden-vector generator and the tests.

Every input is regenerated from (seed, shape, distribution) with numpy's
Philox bit generator, which gives the same numbers on every platform, so a
fixture only needs to store the reference's outputs (or their hashes).

Case matrix (after the reference's own test suites, test/convolve.cpp:36-214:
dtypes x {vector, rectangle, cuboid} x {one2one, many2one, many2many,
one2many} x {EXPAND, DEFAULT}); integer inputs are kept in range so that the
reference's `InT(accum)` conversion is defined.
"""
from __future__ import annotations

import numpy as np

F32, C32, F64, C64, B8, S32, U32, U8, S64, U64, S16, U16, F16, S8 = range(14)
NP_OF = {F32: np.float32, C32: np.complex64, F64: np.float64, C64: np.complex128, B8: np.int8,
         S32: np.int32, U32: np.uint32, U8: np.uint8, S64: np.int64, U64: np.uint64,
         S16: np.int16, U16: np.uint16, S8: np.int8}
ACC_OF = {F32: np.float32, F64: np.float64, C32: np.complex64, C64: np.complex128}
DT_NAME = {F32: "f32", C32: "c32", F64: "f64", C64: "c64", B8: "b8", S32: "s32", U32: "u32",
           U8: "u8", S64: "s64", U64: "u64", S16: "s16", U16: "u16", S8: "s8"}
EIGHT_BIT = (U8, S8, B8)


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(seed))


def af_shape(dims):
    d = list(dims) + [1] * (4 - len(dims))
    return d[:4]


def make_signal(dtype: int, dims, seed: int) -> np.ndarray:
    g = rng(seed)
    shape = af_shape(dims)
    if dtype in (F32, F64):
        a = g.standard_normal(shape)
    elif dtype in (C32, C64):
        a = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    elif dtype == B8:
        a = g.integers(0, 2, shape)
    else:
        a = g.integers(0, 10, shape)
    return np.asfortranarray(a.astype(NP_OF[dtype]))


def make_filter(dtype: int, dims, seed: int, rank: int) -> np.ndarray:
    """Filter in the accumulator type.  Integer signals get non-negative taps
    normalised to unit sum per filter slice so every output stays in range."""
    g = rng(seed)
    shape = af_shape(dims)
    acc = ACC_OF.get(dtype, np.float32)
    if dtype in (F32, F64):
        f = g.standard_normal(shape)
    elif dtype in (C32, C64):
        f = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    else:
        f = g.random(shape) + 0.05
        f = f / f.sum(axis=tuple(range(rank)), keepdims=True)
        if dtype in (S16, U16, S32, U32, S64, U64):
            f = f * 3.0
    return np.asfortranarray(f.astype(acc))


# (name, rank, signal dims, filter dims, kind label)
DIRECT_SHAPES = [
    # rank 1
    ("v_one2one", 1, (37,), (5,)),
    ("v_one2one_even", 1, (37,), (4,)),
    ("v_many2one", 1, (23, 3, 2), (7,)),
    ("v_one2many", 1, (23,), (5, 3)),
    ("v_many2many", 1, (19, 3), (3, 3)),
    # rank 2
    ("r_one2one_3", 2, (33, 21), (3, 3)),
    ("r_one2one_5", 2, (70, 65), (5, 5)),
    ("r_one2one_7", 2, (67, 130), (7, 7)),
    ("r_one2one_2x4", 2, (29, 17), (2, 4)),
    ("r_one2one_9", 2, (31, 40), (9, 9)),
    ("r_one2one_17", 2, (40, 33), (17, 17)),
    ("r_many2one", 2, (45, 38, 3), (5, 5)),
    ("r_many2one_4d", 2, (30, 20, 2, 2), (3, 3)),
    ("r_one2many", 2, (41, 26), (3, 3, 3)),
    ("r_many2many", 2, (66, 70, 3), (7, 7, 3)),
    ("r_small", 2, (3, 2), (5, 5)),
    # widths that are 16-byte multiples for f32 and 8-bit data (TMA-staged path)
    ("r_tma_7_lhs", 2, (128, 96, 3), (7, 7)),
    ("r_tma_5_same", 2, (64, 70, 2), (5, 5, 2)),
    ("r_tma_3_rhs", 2, (96, 33), (3, 3, 2)),
    ("r_tma_7_4d", 2, (64, 65, 2, 2), (7, 7)),
    # rank 3
    ("c_one2one_3", 3, (17, 14, 9), (3, 3, 3)),
    ("c_one2one_245", 3, (11, 13, 10), (2, 4, 5)),
    ("c_many2one", 3, (9, 8, 7, 2), (3, 3, 3)),
    ("c_one2many", 3, (9, 8, 7), (3, 3, 3, 2)),
    ("c_many2many", 3, (9, 8, 7, 2), (3, 3, 3, 2)),
    # 16-byte-multiple widths (TMA-staged 3-D path), every batch kind
    ("c_tma_one", 3, (64, 20, 18), (3, 3, 3)),
    ("c_tma_lhs", 3, (32, 12, 10, 2), (3, 3, 3)),
    ("c_tma_same", 3, (36, 10, 9, 2), (3, 3, 3, 2)),
    ("c_tma_rhs", 3, (40, 9, 11), (3, 3, 3, 2)),
]

DIRECT_DTYPES_FULL = [F32, F64, C32, C64, U8, S8, B8, S16, U16, S32, U32, S64, U64]
DIRECT_DTYPES_SHORT = [F32, F64, C32, U8, S32]


def direct_cases():
    """Yields (case_id, dtype, rank, sig_dims, filt_dims, expand, seed)."""
    seed = 1000
    for name, rank, sd, fd in DIRECT_SHAPES:
        dts = DIRECT_DTYPES_FULL if name in ("r_one2one_5", "r_one2many", "v_many2one",
                                             "c_one2one_3", "r_many2many") else DIRECT_DTYPES_SHORT
        for dt in dts:
            for expand in (False, True):
                seed += 2
                yield (f"{name}_{DT_NAME[dt]}_{'exp' if expand else 'def'}", dt, rank, sd, fd,
                       expand, seed)


SEP_SHAPES = [
    ("sep_5x3", (40, 33), 5, 3),
    ("sep_15", (70, 66, 2), 15, 15),
    ("sep_2x7", (31, 29), 2, 7),
    ("sep_31", (80, 70), 31, 31),
    ("sep_batch4d", (20, 21, 2, 2), 3, 5),
    # 16-byte-multiple widths (TMA-staged path)
    ("sep_15_tma", (128, 80, 2), 15, 15),
    ("sep_3_tma", (64, 50), 3, 3),
    ("sep_7_tma", (96, 70, 3), 7, 7),
]
SEP_DTYPES = [F32, F64, C32, U8, S8, S16, S32, U32, S64]


def sep_taps(dtype: int, n: int, seed: int) -> np.ndarray:
    g = rng(seed)
    acc = ACC_OF.get(dtype, np.float32)
    if dtype in (F32, F64):
        t = g.standard_normal(n)
    elif dtype in (C32, C64):
        t = g.standard_normal(n) + 1j * g.standard_normal(n)
    else:
        # the CPU backend converts taps to the input type (truncation toward
        # zero, src/backend/cpu/kernel/convolve.hpp:233): fractional taps in
        # [0,1) become 0 and two taps in [1,2.5) become 1 or 2, which
        # exercises the rule while keeping every product and sum in range
        t = g.random(n)
        for pos in g.choice(n, size=min(2, n), replace=False):
            t[pos] = 1.0 + 1.5 * g.random()
    return t.astype(acc)


def sep_signal(dtype: int, dims, seed: int) -> np.ndarray:
    g = rng(seed)
    shape = af_shape(dims)
    if dtype in (F32, F64):
        a = g.standard_normal(shape)
    elif dtype in (C32, C64):
        a = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    else:
        a = g.integers(0, 3, shape)
    return np.asfortranarray(a.astype(NP_OF[dtype]))


def sep_cases():
    seed = 5000
    for name, sd, cl, rl in SEP_SHAPES:
        for dt in SEP_DTYPES:
            for expand in (False, True):
                seed += 3
                yield (f"{name}_{DT_NAME[dt]}_{'exp' if expand else 'def'}", dt, sd, cl, rl, expand, seed)


# NN geometry cases: (name, signal dims (W,H,C,N), filter dims (fw,fh,C,K), stride, pad, dil)
NN_CASES = [
    ("nn_s1p1", (10, 10, 1, 1), (3, 3, 1, 1), (1, 1), (1, 1), (1, 1)),
    ("nn_s3p1", (10, 10, 1, 1), (3, 3, 1, 1), (3, 3), (1, 1), (1, 1)),
    ("nn_5x5_s5", (10, 10, 1, 1), (5, 5, 1, 1), (5, 5), (1, 1), (1, 1)),
    ("nn_d2", (10, 10, 1, 1), (3, 3, 1, 1), (1, 1), (1, 1), (2, 2)),
    ("nn_d3", (10, 10, 1, 1), (3, 3, 1, 1), (1, 1), (1, 1), (3, 3)),
    ("nn_35", (10, 10, 1, 1), (3, 5, 1, 1), (1, 1), (1, 1), (1, 1)),
    ("nn_35_s31_d21", (10, 10, 1, 1), (3, 5, 1, 1), (3, 1), (1, 1), (2, 1)),
    ("nn_multi", (8, 10, 3, 2), (3, 3, 3, 4), (1, 1), (1, 1), (1, 1)),
    ("nn_s2_c16", (17, 15, 16, 2), (3, 3, 16, 24), (2, 2), (1, 1), (1, 1)),
    ("nn_5x5_d2_s2", (20, 18, 8, 2), (5, 5, 8, 12), (2, 2), (4, 4), (2, 2)),
    ("nn_1x1", (14, 14, 32, 2), (1, 1, 32, 40), (1, 1), (0, 0), (1, 1)),
    ("nn_nopad", (12, 11, 5, 3), (3, 2, 5, 7), (1, 2), (0, 0), (1, 1)),
]


def nn_inputs(case, seed: int, dtype=np.float32):
    name, sd, fd, st, pd, dl = case
    g = rng(seed)
    s = np.asfortranarray(g.standard_normal(af_shape(sd)).astype(dtype))
    std = np.sqrt(2.0 / (fd[0] * fd[1] * fd[2]))
    f = np.asfortranarray((g.standard_normal(af_shape(fd)) * std).astype(dtype))
    return s, f


def nn_out_dims(sd, fd, st, pd, dl):
    def div(a, b):
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b > 0) else -q
    wo = 1 + div(sd[0] + 2 * pd[0] - ((fd[0] - 1) * dl[0] + 1), st[0])
    ho = 1 + div(sd[1] + 2 * pd[1] - ((fd[1] - 1) * dl[1] + 1), st[1])
    return [wo, ho, fd[3], af_shape(sd)[3]]


def nn_grad(case, seed: int, dtype=np.float32):
    name, sd, fd, st, pd, dl = case
    g = rng(seed + 7)
    od = nn_out_dims(af_shape(sd), af_shape(fd), st, pd, dl)
    return np.asfortranarray(g.standard_normal(od).astype(dtype))


# the two full-size f32 image workloads (512x512 Gaussian blur, 1024x1024 neighbour
# count); outputs stored as SHA-256 of the reference's bytes
def config1a():
    """512x512 f32 U[0,1) (Philox seed 0) with the 5x5 Gaussian sigma=1,
    normalised to unit sum (src/api/c/gaussian_kernel.cpp:36-88)."""
    sig = np.asfortranarray(rng(0).random((512, 512), dtype=np.float32))
    x = np.arange(5) - 2
    k = np.exp(-0.5 * (x[:, None] ** 2 + x[None, :] ** 2) / 1.0 ** 2)
    k = (k / k.sum()).astype(np.float32)
    return sig, np.asfortranarray(k)


def config1b():
    """1024x1024 Bernoulli(0.5) binary f32 grid with the 3x3 all-ones-except-
    centre neighbour kernel (examples/graphics/conway.cpp:18)."""
    sig = np.asfortranarray((rng(1).random((1024, 1024)) < 0.5).astype(np.float32))
    k = np.ones((3, 3), np.float32)
    k[1, 1] = 0
    return sig, np.asfortranarray(k)


# af_unwrap / af_wrap: every type x the reference's geometry families
# (test/unwrap.cpp:104-147, test/wrap.cpp:163-181: window, stride, padding
# combinations on small images), both layouts, two batch slices each way.
PATCH_DTYPES = [F32, C32, F64, C64, B8, S32, U32, U8, S64, U64, S16, U16, S8]
PATCH_GEOMS = [
    # name,    (W, H),  wx, wy, sx, sy, px, py
    ("p3s1",   (13, 9),  3, 3, 1, 1, 0, 0),
    ("p3s1p1", (13, 9),  3, 3, 1, 1, 1, 1),
    ("p3s2p2", (13, 9),  3, 3, 2, 2, 2, 2),
    ("p4s2p3", (16, 10), 4, 4, 2, 2, 3, 3),
    ("p8s8p7", (30, 20), 8, 8, 8, 8, 7, 7),
    ("p8x12",  (30, 20), 8, 12, 8, 12, 7, 11),
    ("p15x10", (30, 20), 15, 10, 1, 1, 14, 9),
    ("p31s8",  (40, 33), 31, 31, 8, 8, 15, 15),
    ("p5r",    (21, 17), 5, 3, 3, 2, 1, 2),
]


def patch_cases():
    """(id, dtype, (W, H, d2, d3), wx, wy, sx, sy, px, py, is_column, seed)."""
    out = []
    seed = 20000
    for gname, (W, H), wx, wy, sx, sy, px, py in PATCH_GEOMS:
        for dt in PATCH_DTYPES:
            for col in (True, False):
                seed += 3
                out.append((f"{gname}_{DT_NAME[dt]}_{'col' if col else 'row'}", dt, (W, H, 2, 2),
                            wx, wy, sx, sy, px, py, col, seed))
    return out


def patch_values(dtype: int, shape, seed: int) -> np.ndarray:
    """Values for unwrap inputs and wrap patch matrices: integers large enough
    that 8- and 16-bit accumulations wrap around."""
    g = rng(seed)
    shape = af_shape(shape)
    if dtype in (F32, F64):
        a = g.standard_normal(shape) * 4
    elif dtype in (C32, C64):
        a = (g.standard_normal(shape) + 1j * g.standard_normal(shape)) * 4
    elif dtype == B8:
        a = g.integers(0, 2, shape)
    elif dtype in (U8, S8):
        a = g.integers(0, 120, shape)
    elif dtype in (S16, U16):
        a = g.integers(0, 30000, shape)
    else:
        a = g.integers(0, 1 << 30, shape)
    return np.asfortranarray(a.astype(NP_OF[dtype]))


def patch_dims(case):
    """unwrap output dims of a patch case."""
    _, _, (W, H, d2, d3), wx, wy, sx, sy, px, py, col, _ = case
    nx = (W + 2 * px - wx) // sx + 1
    ny = (H + 2 * py - wy) // sy + 1
    return [wx * wy, nx * ny, d2, d3] if col else [nx * ny, wx * wy, d2, d3]


# af_sobel_operator: every accepted type on images, batches and small sizes
SOBEL_DTYPES = [F32, F64, S32, U32, S16, U16, B8, S8, U8]
SOBEL_SHAPES = [(17, 13), (16, 9, 3), (2, 2), (64, 3, 2, 2), (3, 40)]


def sobel_cases():
    out = []
    seed = 30000
    for shape in SOBEL_SHAPES:
        for dt in SOBEL_DTYPES:
            seed += 1
            out.append((f"sobel_{'x'.join(map(str, shape))}_{DT_NAME[dt]}", dt, shape, seed))
    return out


def sobel_input(dt: int, shape, seed: int) -> np.ndarray:
    x = make_signal(dt, shape, seed)
    if dt in (F32, F64):
        x = (x * 10).astype(x.dtype)
    return np.asfortranarray(x)


# ---------------------------------------------------------------------------
# af_harris: (id, dtype, (d0, d1), max_corners, min_response, sigma,
# block_size, k_thr, image kind, seed).  "blocks" are bright rectangles on
# a dark ground plus faint noise, scaled to [0, 255]; "tiles" repeat one
# random 12x12 tile exactly, so many corners tie on score (the sort's
# stability decides their order); "noise" is smoothed random texture.
# ---------------------------------------------------------------------------
def harris_cases():
    base = [
        ("mc500_default", (64, 48), 500, 1e5, 1.0, 0, 0.04, "blocks"),
        ("mc20_sorted", (100, 80), 20, 0.0, 1.0, 0, 0.04, "blocks"),
        ("minresp_sigma2", (97, 131), 0, 1000.0, 2.0, 0, 0.06, "blocks"),
        ("box5_sorted", (64, 64), 10, 0.0, 0.3, 5, 0.04, "blocks"),
        ("block7_gauss", (120, 90), 0, 50.0, 1.5, 7, 0.05, "blocks"),
        ("sigma5_len29", (160, 150), 10, 0.0, 5.0, 0, 0.04, "noise"),
        ("block32_box", (180, 140), 0, 10.0, 0.2, 32, 0.04, "noise"),
        ("ties_sorted", (120, 96), 25, 0.0, 1.0, 0, 0.04, "tiles"),
        ("ties_all", (96, 120), 0, 1.0, 1.0, 3, 0.04, "tiles"),
        ("one_interior_px", (9, 9), 10, 0.0, 1.0, 0, 0.04, "noise"),
        ("too_narrow", (8, 40), 10, 0.0, 1.0, 0, 0.04, "noise"),
        ("noise_many", (257, 190), 0, 0.5, 1.0, 0, 0.04, "noise"),
    ]
    out = []
    seed = 40000
    for name, shape, mc, mr, sg, bs, k, kind in base:
        for dt in (F32, F64):
            seed += 1
            out.append((f"harris_{name}_{DT_NAME[dt]}", dt, shape, mc, mr, sg, bs, k, kind, seed))
    return out


def harris_image(dt: int, shape, kind: str, seed: int) -> np.ndarray:
    g = rng(seed)
    d0, d1 = shape
    if kind == "tiles":
        tile = g.random((12, 12)) * 255.0
        a = np.tile(tile, (d0 // 12 + 1, d1 // 12 + 1))[:d0, :d1]
    elif kind == "noise":
        a = g.random((d0 + 4, d1 + 4))
        a = (a[:-4, :-4] + a[2:-2, 2:-2] + a[4:, 4:] + a[4:, :-4]) * 64.0
    else:
        y, x = np.mgrid[0:d0, 0:d1]
        a = np.zeros((d0, d1))
        for _ in range(20):
            cy, cx = g.uniform(0, d0), g.uniform(0, d1)
            w = g.uniform(3, 12)
            a += ((np.abs(y - cy) < w) & (np.abs(x - cx) < w * 1.3)) * g.uniform(0.3, 1.0)
        a = a * 200.0 + 5.0 * g.standard_normal((d0, d1))
    return np.asfortranarray(a.astype(NP_OF[dt]))


# ---------------------------------------------------------------------------
# af_canny: (id, dtype, dims, otsu, low ratio, high ratio, is_fast, image
# kind, seed).  Images as for Harris; integer types get the image clipped to
# their range.  "wide" shapes (d1 > d0 + 3) exercise the reference's seed
# scan, which stops before the last columns.
# ---------------------------------------------------------------------------
CANNY_TYPES = (F32, F64, S32, U32, S16, U16, S8, U8)


def canny_cases():
    base = [
        ("manual_l2", (64, 48), False, 0.1, 0.3, False, "blocks"),
        ("otsu_l2", (100, 80), True, 0.4, 0.0, False, "blocks"),
        ("manual_l1_wide", (97, 131), False, 0.05, 0.2, True, "noise"),
        ("otsu_l1_tiles", (120, 90), True, 0.3, 0.0, True, "tiles"),
        ("manual_batch3", (60, 60, 3), False, 0.1, 0.25, False, "blocks"),
        ("manual_very_wide", (40, 150), False, 0.08, 0.3, False, "blocks"),
        ("otsu_batch2", (70, 64, 2), True, 0.5, 0.0, False, "blocks"),
        ("smallest_5x5", (5, 5), False, 0.1, 0.2, False, "noise"),
    ]
    out = []
    seed = 50000
    for name, shape, otsu, t1, t2, isf, kind in base:
        for dt in CANNY_TYPES:
            seed += 1
            out.append((f"canny_{name}_{DT_NAME[dt]}", dt, shape, otsu, t1, t2, isf, kind, seed))
    return out


def canny_image(dt: int, shape, kind: str, seed: int) -> np.ndarray:
    planes = [harris_image(F64, shape[:2], kind, seed + 1000 * z)
              for z in range(shape[2] if len(shape) > 2 else 1)]
    a = np.stack(planes, axis=2) if len(planes) > 1 else planes[0]
    if dt == S8:
        a = np.clip(a * 0.5, -128, 127)
    elif dt not in (F32, F64):
        a = np.clip(a, 0, 255)
    return np.asfortranarray(a.astype(NP_OF[dt]))
