"""Python face of the oracle — TEST INFRASTRUCTURE ONLY (the checker, never the
thing measured or shipped).

Two implementations sit behind the same functions:

* ``port``: ``conv_oracle.c``, a plain-C restatement of ArrayFire's CPU
  convolution loops (built by ``make -C oracle port``; builds on any host);
* ``ref``:  the reference's own CPU kernel templates compiled in place
  (``make -C oracle ref``; only where an ArrayFire source tree is present).

Arrays follow ArrayFire's layout: a numpy array of shape (d0, d1, d2, d3) in
Fortran (column-major) order, so element (i,j,k,l) sits at
i + d0*(j + d1*(k + d2*l)), exactly as ``af::array``.

Host dispatch logic restated here (same decisions as the library):
  identify_batch_kind  src/api/c/convolve.cpp:77-97
  conv_output_dims     src/backend/cpu/convolve.cpp:38-58
  nn_output_dims       src/backend/cpu/convolve.cpp:130-135
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libafref.so"

# af_dtype numbering (include/af/defines.h:211-233)
F32, C32, F64, C64, B8, S32, U32, U8, S64, U64, S16, U16, F16, S8 = range(14)
NP_OF = {
    F32: np.float32, C32: np.complex64, F64: np.float64, C64: np.complex128,
    B8: np.int8, S32: np.int32, U32: np.uint32, U8: np.uint8, S64: np.int64,
    U64: np.uint64, S16: np.int16, U16: np.uint16, F16: np.float16, S8: np.int8,
}
ACC_OF = {F32: np.float32, F64: np.float64, C32: np.complex64, C64: np.complex128}
BATCH_NONE, BATCH_LHS, BATCH_RHS, BATCH_SAME, BATCH_DIFF, BATCH_UNSUPPORTED = range(6)

_P = ctypes.c_void_p
_LL4 = ctypes.POINTER(ctypes.c_longlong)


def acc_np(dtype: int):
    return ACC_OF.get(dtype, np.float32)


def build_port() -> Path:
    """Compile conv_oracle.c (gcc) if needed."""
    src = HERE / "conv_oracle.c"
    if not PORT_LIB.exists() or PORT_LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_LIB


def build_ref(reference: str | None = None) -> Path | None:
    """Compile the reference's CPU kernels in place, when its tree exists."""
    # AF_REFERENCE_SRC, else an ArrayFire checkout named `reference` beside this repository
    ref = reference or os.environ.get("AF_REFERENCE_SRC") or str(HERE.parent.parent / "reference")
    if not Path(ref, "src", "backend", "cpu", "kernel", "convolve.hpp").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REFERENCE={ref}"], check=True)
    return REF_LIB


_libs: dict[str, ctypes.CDLL] = {}


def lib(which: str = "port") -> ctypes.CDLL:
    if which not in _libs:
        if which == "port":
            path = build_port()
        elif which == "ref":
            if not REF_LIB.exists():
                raise FileNotFoundError("oracle/_ref/libafref.so not built (needs the reference tree)")
            path = REF_LIB
        else:
            raise ValueError(which)
        _libs[which] = ctypes.CDLL(str(path))
    return _libs[which]


def have_ref() -> bool:
    return REF_LIB.exists()


def _ll(vals) -> ctypes.Array:
    return (ctypes.c_longlong * len(vals))(*[int(v) for v in vals])


def _dims4(a: np.ndarray) -> list[int]:
    d = list(a.shape) + [1] * (4 - a.ndim)
    return d[:4]


def _dense_strides(d) -> list[int]:
    return [1, d[0], d[0] * d[1], d[0] * d[1] * d[2]]


def as_af(a: np.ndarray, dtype=None) -> np.ndarray:
    """Reshape to 4-D column-major (copying when needed)."""
    a = np.asarray(a, dtype=dtype)
    d = _dims4(a)
    return np.asfortranarray(a.reshape(d, order="F"))


def ndims(d) -> int:
    """af::dim4::ndims (src/backend/common/dim4.cpp:48-58)."""
    d = list(d) + [1] * (4 - len(d))
    n = d[0] * d[1] * d[2] * d[3]
    if n == 0:
        return 0
    if n == 1:
        return 1
    for i in (3, 2, 1):
        if d[i] != 1:
            return i + 1
    return 1


def identify_batch_kind(rank: int, sd, fd) -> int:
    sn, fn = ndims(sd), ndims(fd)
    if sn == rank and fn == rank:
        return BATCH_NONE
    if sn == rank and rank < fn <= 4:
        return BATCH_RHS
    if rank < sn <= 4 and fn == rank:
        return BATCH_LHS
    if rank < sn <= 4 and rank < fn <= 4:
        match = all(sd[i] == fd[i] for i in range(rank, 4))
        inter = all(sd[i] == 1 or fd[i] == 1 or sd[i] == fd[i] for i in range(rank, 4))
        if match:
            return BATCH_SAME
        return BATCH_DIFF if inter else BATCH_UNSUPPORTED
    return BATCH_UNSUPPORTED


def conv_output_dims(rank, kind, expand, sd, fd):
    if expand:
        if kind in (BATCH_NONE, BATCH_RHS):
            return [sd[d] + fd[d] - 1 for d in range(4)]
        return [sd[d] + fd[d] - 1 if d < rank else sd[d] for d in range(4)]
    od = list(sd)
    if kind == BATCH_RHS:
        for i in range(rank, 4):
            od[i] = fd[i]
    return od


def _cdiv_trunc(a: int, b: int) -> int:
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def nn_output_dims(sd, fd, stride, pad, dil):
    wo = 1 + _cdiv_trunc(sd[0] + 2 * pad[0] - ((fd[0] - 1) * dil[0] + 1), stride[0])
    ho = 1 + _cdiv_trunc(sd[1] + 2 * pad[1] - ((fd[1] - 1) * dil[1] + 1), stride[1])
    return [wo, ho, fd[3], sd[3]]


# ---------------------------------------------------------------------------
# direct convolutions
# ---------------------------------------------------------------------------
def convolve(sig: np.ndarray, filt: np.ndarray, dtype: int, rank: int, expand: bool,
             which: str = "port") -> np.ndarray:
    """af_convolve{1,2,3} in the spatial domain: dispatch exactly like
    src/api/c/convolve.cpp:132-215 then run convolve_nd."""
    s = as_af(sig, NP_OF[dtype])
    f = as_af(filt, acc_np(dtype))
    sd, fd = _dims4(s), _dims4(f)
    kind = identify_batch_kind(rank, sd, fd)
    if kind in (BATCH_DIFF, BATCH_UNSUPPORTED):
        raise ValueError("unsupported batch kind")
    od = conv_output_dims(rank, kind, expand, sd, fd)
    out = np.zeros(od, dtype=NP_OF[dtype], order="F")
    fn = lib(which).oracle_convolve_nd if which == "port" else lib(which).ref_convolve_nd
    rc = fn(ctypes.c_int(dtype), out.ctypes.data_as(_P), _ll(od), _ll(_dense_strides(od)),
            s.ctypes.data_as(_P), _ll(sd), _ll(_dense_strides(sd)), f.ctypes.data_as(_P),
            _ll(fd), _ll(_dense_strides(fd)), ctypes.c_int(kind), ctypes.c_int(rank),
            ctypes.c_int(1 if expand else 0))
    if rc != 0:
        raise RuntimeError(f"oracle convolve failed ({rc})")
    return out


def convolve2_sep(sig: np.ndarray, cfilt: np.ndarray, rfilt: np.ndarray, dtype: int,
                  expand: bool, which: str = "port") -> np.ndarray:
    """af_convolve2_sep (src/api/c/convolve.cpp:258-334 ->
    src/backend/cpu/convolve.cpp:68-99)."""
    s = as_af(sig, NP_OF[dtype])
    c = np.ascontiguousarray(np.asarray(cfilt, dtype=acc_np(dtype)).ravel(order="F"))
    r = np.ascontiguousarray(np.asarray(rfilt, dtype=acc_np(dtype)).ravel(order="F"))
    sd = _dims4(s)
    od = list(sd)
    if expand:
        od[0] += c.size - 1
        od[1] += r.size - 1
    out = np.zeros(od, dtype=NP_OF[dtype], order="F")
    fn = lib(which).oracle_convolve2_sep if which == "port" else lib(which).ref_convolve2_sep
    rc = fn(ctypes.c_int(dtype), out.ctypes.data_as(_P), _ll(od), s.ctypes.data_as(_P), _ll(sd),
            c.ctypes.data_as(_P), ctypes.c_longlong(c.size), r.ctypes.data_as(_P),
            ctypes.c_longlong(r.size), ctypes.c_int(1 if expand else 0))
    if rc != 0:
        raise RuntimeError(f"oracle convolve2_sep failed ({rc})")
    return out


# ---------------------------------------------------------------------------
# unwrap / wrap
# ---------------------------------------------------------------------------
def unwrap(sig: np.ndarray, wx, wy, sx, sy, px, py, dx, dy, which="port") -> np.ndarray:
    s = as_af(sig)
    t = s.dtype
    assert t in (np.float32, np.float64)
    sd = _dims4(s)
    nx = 1 + _cdiv_trunc(sd[0] + 2 * px - ((wx - 1) * dx + 1), sx)
    ny = 1 + _cdiv_trunc(sd[1] + 2 * py - ((wy - 1) * dy + 1), sy)
    out = np.zeros([wx * wy, nx * ny, sd[2], sd[3]], dtype=t, order="F")
    suffix = "f32" if t == np.float32 else "f64"
    name = ("oracle_unwrap_" if which == "port" else "ref_unwrap_") + suffix
    getattr(lib(which), name)(out.ctypes.data_as(_P), s.ctypes.data_as(_P), _ll(sd),
                              *[ctypes.c_longlong(v) for v in (wx, wy, sx, sy, px, py, dx, dy)])
    return out


def wrap_dilated(cols: np.ndarray, odims, wx, wy, sx, sy, px, py, dx, dy, which="port"):
    c = as_af(cols)
    t = c.dtype
    out = np.zeros(list(odims), dtype=t, order="F")
    suffix = "f32" if t == np.float32 else "f64"
    name = ("oracle_wrap_dilated_" if which == "port" else "ref_wrap_dilated_") + suffix
    getattr(lib(which), name)(out.ctypes.data_as(_P), _ll(odims), c.ctypes.data_as(_P),
                              *[ctypes.c_longlong(v) for v in (wx, wy, sx, sy, px, py, dx, dy)])
    return out


# ---------------------------------------------------------------------------
# af_fft_convolve1/2/3 (frequency-domain semantics)
# ---------------------------------------------------------------------------
def _round_half_away(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def fft_convolve(sig: np.ndarray, filt: np.ndarray, dtype: int, rank: int, expand: bool):
    """What the reference's frequency-domain path returns, computed exactly in
    FP64 (src/api/c/fftconvolve.cpp:38-152 and src/backend/cpu/fftconvolve.cpp:
    38-200, kernel/fftconvolve.hpp:179-250):

    * real signal, batch kind NONE/LHS/RHS/SAME: the filter is converted to
      the signal type first (castArray<T>: integer signals truncate the taps);
      integer outputs are rounded half away from zero (roundf);
    * complex signal or DIFF batch (fftconvolve_fallback): the filter keeps its
      values; the real part (complex value) is converted without rounding;
    * EXPAND: the full s+f-1 window of the rank dims, DEFAULT: from f//2;
      batch dims max(s, f).
    The linear convolution itself is exact here (FP64); the library's FP32
    transforms agree within rounding."""
    s = as_af(sig)
    f = as_af(filt)
    sd, fd = _dims4(s), _dims4(f)
    kind = identify_batch_kind(rank, sd, fd)
    if kind == BATCH_UNSUPPORTED:
        raise ValueError("unsupported batch")
    t = NP_OF[dtype]
    cplx = dtype in (C32, C64)
    fallback = cplx or kind == BATCH_DIFF
    if not fallback:
        # castArray<T>: C conversion, truncating toward zero; b8 is (v != 0)
        # (src/backend/cpu/cast.hpp:140-155)
        f = (f != 0).astype(t) if dtype == B8 else f.astype(t)
    sw = s.astype(np.complex128 if cplx else np.float64)
    fw = f.astype(np.complex128 if (cplx or np.iscomplexobj(f)) else np.float64)
    full = [sd[k] + fd[k] - 1 for k in range(rank)]
    axes = tuple(range(rank))
    Sf = np.fft.fftn(sw, s=full, axes=axes)
    Ff = np.fft.fftn(fw, s=full, axes=axes)
    # broadcast batch dims (each is 1 on one side or equal)
    res = np.fft.ifftn(Sf * Ff, axes=axes)
    if not (cplx or np.iscomplexobj(fw)):
        res = res.real
    elif not cplx:
        res = res.real
    sl = []
    for k in range(4):
        if k < rank:
            sl.append(slice(0, full[k]) if expand else slice(fd[k] // 2, fd[k] // 2 + sd[k]))
        else:
            sl.append(slice(None))
    res = res[tuple(sl)]
    if dtype in (F32, F64, C32, C64):
        out = res.astype(t)
    elif fallback:
        out = np.trunc(res).astype(t)
    else:
        out = _round_half_away(res).astype(t)
    return np.asfortranarray(out)


# ---------------------------------------------------------------------------
# image-processing callers: af_gaussian_kernel, af_dog, af_sobel_operator
# ---------------------------------------------------------------------------
SOBEL_OUT = {F32: F32, F64: F64, S32: S32, U32: S32, S16: S32, U16: S32, B8: S32, S8: S32,
             U8: S32}


def gaussian_kernel(rows: int, cols: int, sigma_r: float = 0.0, sigma_c: float = 0.0):
    """src/api/c/gaussian_kernel.cpp:29-88, in FP64: exp(-((j - (cols-1)/2)/sc)^2/2
    - ((i - (rows-1)/2)/sr)^2/2) normalised to unit sum, sc = sigma_c or cols/4."""
    i = np.arange(rows, dtype=np.float64)[:, None]
    j = np.arange(cols, dtype=np.float64)[None, :]
    tmp = np.zeros((rows, cols))
    if cols > 1:
        sc = sigma_c if sigma_c > 0 else 0.25 * cols
        tmp = tmp + ((j - (cols - 1) / 2.0) / sc) ** 2
    if rows > 1:
        sr = sigma_r if sigma_r > 0 else 0.25 * rows
        tmp = tmp + ((i - (rows - 1) / 2.0) / sr) ** 2
    g = np.exp(-0.5 * tmp)
    return np.asfortranarray(g / g.sum())


def dog(img: np.ndarray, dtype: int, r1: int, r2: int):
    """src/api/c/dog.cpp:30-54: convolve2 DEFAULT with the two Gaussians in the
    accumulator type (f64 for f64, else f32), then the difference."""
    acc = F64 if dtype == F64 else F32
    x = as_af(img).astype(NP_OF[acc])
    # af_gaussian_kernel is always f32 (gaussian_kernel.cpp:90-99), cast after
    g1 = gaussian_kernel(2 * r1 + 1, 2 * r1 + 1).astype(np.float32).astype(NP_OF[acc])
    g2 = gaussian_kernel(2 * r2 + 1, 2 * r2 + 1).astype(np.float32).astype(NP_OF[acc])
    a = convolve(np.asfortranarray(x), np.asfortranarray(g1), acc, 2, False)
    b = convolve(np.asfortranarray(x), np.asfortranarray(g2), acc, 2, False)
    return np.asfortranarray(a - b)


def _reflect101(idx, end):
    return np.abs(end - np.abs(end - idx)) if end > 0 else np.zeros_like(idx)


def sobel(img: np.ndarray, dtype: int, which: str = "port"):
    """af_sobel_operator, ker_size 3 (src/backend/cpu/kernel/sobel.hpp:19-75):
    returns (dx, dy) in the output type, each operation rounded in the
    reference's order."""
    a = as_af(img)
    d = _dims4(a)
    ot = NP_OF[SOBEL_OUT[dtype]]
    if which == "ref":
        dx = np.zeros(d, dtype=ot, order="F")
        dy = np.zeros(d, dtype=ot, order="F")
        rc = lib("ref").ref_sobel(ctypes.c_int(dtype), dx.ctypes.data_as(_P),
                                  dy.ctypes.data_as(_P), a.ctypes.data_as(_P), _ll(d))
        if rc != 0:
            raise RuntimeError("ref_sobel failed")
        return dx, dy
    x = a.astype(ot)
    i = np.arange(d[0])
    j = np.arange(d[1])
    im, ip = _reflect101(i - 1, d[0] - 1), _reflect101(i + 1, d[0] - 1)
    jm, jp = _reflect101(j - 1, d[1] - 1), _reflect101(j + 1, d[1] - 1)

    def at(ii, jj):
        return x[ii][:, jj]

    NW, SW, NE, SE = at(im, jm), at(ip, jm), at(im, jp), at(ip, jp)
    N, S, W, E = at(im, j), at(ip, j), at(i, jm), at(i, jp)
    two = ot(2)
    with np.errstate(over="ignore"):
        dx = ((SW + SE) - (NW + NE)) + two * (S - N)
        dy = ((NE + SE) - (NW + SW)) + two * (E - W)
    return np.asfortranarray(dx.astype(ot)), np.asfortranarray(dy.astype(ot))


# ---------------------------------------------------------------------------
# af_harris (src/api/c/harris.cpp:42-95 -> src/backend/cpu/harris.cpp:28-144)
# ---------------------------------------------------------------------------
def harris_filter_len(sigma: float, block_size: int) -> int:
    """src/api/c/harris.cpp:47-50: block_size, else floor(6*sigma) made odd
    (6.f * sigma in float)."""
    if block_size:
        return int(block_size)
    fl = int(math.floor(float(np.float32(6.0) * np.float32(sigma))))
    return fl - 1 if fl % 2 == 0 else fl


def harris_window(filter_len: int, sigma: float, dtype: int) -> np.ndarray:
    """The window of src/backend/cpu/harris.cpp:38-47: a box of 1/filter_len
    when sigma < 0.5, else gaussian1D (src/backend/cpu/utility.hpp:35-49:
    each tap evaluated in double, stored in T, summed in T in order, divided
    in T)."""
    T = NP_OF[dtype]
    if np.float32(sigma) < np.float32(0.5):
        return np.full(filter_len, T(1) / T(filter_len), dtype=T)
    s = float(np.float32(sigma))
    taps = np.zeros(filter_len, dtype=T)
    total = T(0)
    for i in range(filter_len):
        x = i - (filter_len - 1) // 2
        el = T(1.0 / math.sqrt(2 * math.pi * s * s) * math.exp(-((x * x) / (2 * (s * s)))))
        taps[i] = el
        total = T(total + el)
    return (taps / total).astype(T)


def harris(img: np.ndarray, dtype: int, max_corners: int, min_response: float, sigma: float,
           block_size: int, k_thr: float, which: str = "port"):
    """af_harris on a 2-D f32/f64 image: returns (x, y, score) float32 vectors
    (x along dim1, y along dim0), in the reference's order.

    Port of src/backend/cpu/harris.cpp:28-144 with the kernels of
    src/backend/cpu/kernel/gradient.hpp:18-80 (central differences, one-sided
    at the edges) and src/backend/cpu/kernel/harris.hpp:18-118 (products,
    responses det - k*tr^2 on [border, d - border), strict 8-neighbour maxima
    on [border+1, d - border - 1) in scan order, at most 20% of the pixels
    kept); the window is the separable convolve2 of this oracle; with
    max_corners > 0 and more corners found, a stable descending sort by score
    keeps the first max_corners."""
    a = as_af(img, NP_OF[dtype])
    d0, d1 = a.shape[0], a.shape[1]
    T = NP_OF[dtype]
    fl = harris_filter_len(sigma, block_size)
    if which == "ref":
        cap = max(int(np.float32(d0 * d1) * np.float32(0.2)), 1)
        xo = np.zeros(cap, np.float32)
        yo = np.zeros(cap, np.float32)
        ro = np.zeros(cap, np.float32)
        n = lib("ref").ref_harris(ctypes.c_int(dtype), a.ctypes.data_as(_P), ctypes.c_longlong(d0),
                                  ctypes.c_longlong(d1), ctypes.c_uint(max_corners),
                                  ctypes.c_float(min_response), ctypes.c_float(sigma),
                                  ctypes.c_uint(fl), ctypes.c_float(k_thr), xo.ctypes.data_as(_P),
                                  yo.ctypes.data_as(_P), ro.ctypes.data_as(_P),
                                  ctypes.c_longlong(cap))
        if n < 0:
            raise RuntimeError(f"ref_harris failed ({n})")
        return xo[:n].copy(), yo[:n].copy(), ro[:n].copy()
    x = a[:, :, 0, 0]
    border = fl // 2 + 1
    r = border + 1
    empty = (np.zeros(0, np.float32),) * 3
    if d0 <= 2 * r or d1 <= 2 * r:
        return empty
    # gradient(iy, ix, in): grad0 along dim0 is iy, grad1 along dim1 is ix
    iy = np.empty_like(x)
    ix = np.empty_like(x)
    half = T(0.5)
    iy[1:-1, :] = half * (x[2:, :] - x[:-2, :])
    iy[0, :] = x[1, :] - x[0, :]
    iy[-1, :] = x[-1, :] - x[-2, :]
    ix[:, 1:-1] = half * (x[:, 2:] - x[:, :-2])
    ix[:, 0] = x[:, 1] - x[:, 0]
    ix[:, -1] = x[:, -1] - x[:, -2]
    win = harris_window(fl, sigma, dtype)
    ixx = convolve2_sep(np.asfortranarray(ix * ix), win, win, dtype, False)[:, :, 0, 0]
    ixy = convolve2_sep(np.asfortranarray(ix * iy), win, win, dtype, False)[:, :, 0, 0]
    iyy = convolve2_sep(np.asfortranarray(iy * iy), win, win, dtype, False)[:, :, 0, 0]
    k = T(np.float32(k_thr))
    resp = np.zeros((d0, d1), T)
    sl = (slice(border, d0 - border), slice(border, d1 - border))
    tr = ixx[sl] + iyy[sl]
    det = ixx[sl] * iyy[sl] - ixy[sl] * ixy[sl]
    resp[sl] = det - k * (tr * tr)
    v = resp[r:d0 - r, r:d1 - r]
    mx = None
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            if dy == 0 and dx == 0:
                continue
            nb = resp[r + dy:d0 - r + dy, r + dx:d1 - r + dx]
            mx = nb if mx is None else np.maximum(mx, nb)
    min_r = 0 if max_corners > 0 else int(np.float32(min_response))
    keep = (v > mx) & (v >= T(np.float32(min_r)))
    idx = np.flatnonzero(keep.ravel(order="F"))
    h = d0 - 2 * r
    ys = (idx % h + r).astype(np.float32)
    xs = (idx // h + r).astype(np.float32)
    sc = v.ravel(order="F")[idx].astype(np.float32)
    corner_lim = int(np.float32(d0 * d1) * np.float32(0.2))
    found = idx.size
    ys, xs, sc = ys[:corner_lim], xs[:corner_lim], sc[:corner_lim]
    out_n = min(found, max_corners if max_corners > 0 else corner_lim)
    if max_corners > 0 and found > out_n:
        order = np.argsort(-sc, kind="stable")[:out_n]
        return xs[order], ys[order], sc[order]
    return xs[:out_n], ys[:out_n], sc[:out_n]


# ---------------------------------------------------------------------------
# af_canny (src/api/c/canny.cpp:196-285; CPU kernels src/backend/cpu/kernel/canny.hpp)
# ---------------------------------------------------------------------------
CANNY_TYPES = (F32, F64, S32, U32, S16, U16, S8, U8)
CANNY_TAPS = np.array([-0.11021, -0.23691, -0.30576, -0.23691, -0.11021], np.float32)


def canny_nms(mag, gx, gy):
    """kernel::nonMaxSuppression (src/backend/cpu/kernel/canny.hpp:18-116) on
    (d0, d1) float32 planes: interior pixels only; the magnitude interpolated
    along the gradient, each operation rounded separately."""
    d0, d1 = mag.shape
    out = np.zeros_like(mag)
    if d0 < 3 or d1 < 3:
        return out
    c = mag[1:-1, 1:-1]
    se, nw = mag[2:, 2:], mag[:-2, :-2]        # offset +d0+1, -d0-1
    ea, we = mag[2:, 1:-1], mag[:-2, 1:-1]     # offset +1, -1
    ne, sw = mag[2:, :-2], mag[:-2, 2:]        # offset -d0+1, +d0-1
    no, so = mag[1:-1, :-2], mag[1:-1, 2:]     # offset -d0, +d0
    dx, dy = gx[1:-1, 1:-1], gy[1:-1, 1:-1]
    with np.errstate(all="ignore"):
        px, py = dx >= 0, dy >= 0
        g1 = (dx - dy) >= 0          # dx >= 0, dy >= 0
        g2 = (dx + dy) >= 0          # mixed signs
        g4 = (-dx + dy) >= 0         # dx < 0, dy < 0
        q1 = px & py
        q2 = px & ~py
        q3 = ~px & py
        q4 = ~px & ~py
        a1 = np.select([q1, q2, q3, q4], [np.where(g1, ea, so), np.where(g2, ea, no),
                                          np.where(g2, so, we), np.where(g4, we, no)])
        a2 = np.select([q1, q2, q3, q4], [np.where(g1, we, no), np.where(g2, we, so),
                                          np.where(g2, no, ea), np.where(g4, ea, so)])
        b1 = np.select([q1, q2, q3, q4], [se, ne, sw, nw])
        b2 = np.select([q1, q2, q3, q4], [nw, sw, ne, se])
        al = np.select([q1, q2, q3, q4], [np.where(g1, dy / dx, dx / dy),
                                          np.where(g2, -dy / dx, dx / -dy),
                                          np.where(g2, -dx / dy, dy / -dx),
                                          np.where(g4, dy / dx, dx / dy)]).astype(np.float32)
        one = np.float32(1.0)
        m1 = (one - al) * a1 + al * b1
        m2 = (one - al) * a2 + al * b2
        keep = (c != 0) & (c > m1) & (c > m2)
    out[1:-1, 1:-1] = np.where(keep, c, np.float32(0))
    return out


def canny_hysteresis(strong, weak):
    """kernel::edgeTrackingHysteresis (src/backend/cpu/kernel/canny.hpp:148-182)
    on one (d0, d1) slice: seeds are strong pixels at linear indices
    [d0+1, d0 + (d0-1)(d1-1)] (the reference's scan, whose index advances one
    less than a column per column); from each, weak pixels are followed
    through the 8 linear-offset neighbours (t +- 1, t +- d0, t +- d0 +- 1).
    Neighbours outside the slice, which the reference would read out of
    bounds, are skipped."""
    from collections import deque
    d0, d1 = strong.shape
    n = d0 * d1
    s = strong.ravel(order="F") > 0
    w = weak.ravel(order="F") > 0
    out = np.zeros(n, np.int8)
    lo, hi = d0 + 1, d0 + (d0 - 1) * (d1 - 1)
    offs = (-d0 - 1, -d0, -d0 + 1, -1, 1, d0 - 1, d0, d0 + 1)
    for t in np.flatnonzero(s[lo:hi + 1]) + lo:
        if out[t] == 1:
            continue
        out[t] = 1
        q = deque([int(t)])
        while q:
            u = q.popleft()
            for o in offs:
                v = u + o
                if 0 <= v < n and w[v] and out[v] != 1:
                    out[v] = 1
                    q.append(v)
    return out.reshape((d0, d1), order="F")


def canny(img: np.ndarray, dtype: int, otsu: bool, t1: float, t2: float, is_fast: bool,
          which: str = "port") -> np.ndarray:
    """af_canny, sobel window 3, on 2-D slices stacked along dim2: returns an
    int8 (d0, d1, d2) array of 0/1 edges.

    Port of cannyHelper (src/api/c/canny.cpp:205-230): the image cast to
    float, the 5-tap separable smoothing (this oracle's convolve2_sep), the
    Sobel derivatives (this oracle's sobel), |gx| + |gy| or
    sqrt(gx^2 + gy^2), non-maximum suppression, then computeCandidates
    (canny.cpp:153-190): manual thresholds on (s - min) / (max - min), or the
    Otsu threshold of a (max)-bin histogram per slice (otsuThreshold,
    canny.cpp:81-141, every float operation in its order), and hysteresis."""
    a = as_af(img, NP_OF[dtype])
    d = _dims4(a)
    if which == "ref":
        out = np.zeros(d, np.int8, order="F")
        rc = lib("ref").ref_canny(ctypes.c_int(dtype), a.ctypes.data_as(_P), _ll(d),
                                  ctypes.c_int(1 if otsu else 0), ctypes.c_float(t1),
                                  ctypes.c_float(t2), ctypes.c_int(1 if is_fast else 0),
                                  out.ctypes.data_as(_P))
        if rc != 0:
            raise RuntimeError(f"ref_canny failed ({rc})")
        return out[:, :, :, 0]
    x = np.asfortranarray(a.astype(np.float32))
    smt = convolve2_sep(x, CANNY_TAPS, CANNY_TAPS, F32, False)
    gx, gy = sobel(smt, F32)
    if is_fast:
        mag = np.abs(gx) + np.abs(gy)
    else:
        mag = np.sqrt(gx * gx + gy * gy)
    d0, d1, d2 = d[0], d[1], d[2]
    sup = np.zeros((d0, d1, d2), np.float32, order="F")
    for z in range(d2):
        sup[:, :, z] = canny_nms(mag[:, :, z, 0], gx[:, :, z, 0], gy[:, :, z, 0])
    max_v = np.float32(sup.max())
    if otsu:
        nb = int(max_v)
        if nb < 2:
            raise ValueError("the Otsu threshold needs at least two bins")
        step = np.float32(float(max_v) / float(np.float32(nb)))
        total = np.float32(d0 * d1)
        weak = np.zeros_like(sup, dtype=bool)
        strong = np.zeros_like(sup, dtype=bool)
        for z in range(d2):
            v = sup[:, :, z].ravel(order="F")
            with np.errstate(all="ignore"):
                bins = np.clip(((v - np.float32(0)) / step).astype(np.int64), 0, nb - 1)
            hist = np.bincount(bins, minlength=nb)
            freqs = hist.astype(np.float32) / total
            cum = np.add.accumulate(freqs, dtype=np.float32)
            prod = np.arange(nb, dtype=np.float32) * freqs
            cprod = np.add.accumulate(prod, dtype=np.float32)
            ws = cprod[-1]
            best, loc = np.float32(0), 0
            with np.errstate(all="ignore"):
                qL = cum[:-1]
                qH = np.float32(1) - qL
                muL = cprod[:-1] / qL
                muH = (ws - cprod[:-1]) / qH
                diff = muL - muH
                sig = (diff * diff) * (cum[:-1] * (np.float32(1) - cum[:-1]))
            for b in range(nb - 1):  # ireduce<af_max_t>: first maximum, NaN skipped
                if b == 0:
                    best = np.float32(-np.inf) if np.isnan(sig[0]) else sig[0]
                elif sig[b] > best:
                    best, loc = sig[b], b
            T2 = np.float32(loc)
            T1 = T2 * np.float32(t1)
            weak[:, :, z] = (sup[:, :, z] >= T1) & (sup[:, :, z] < T2)
            strong[:, :, z] = sup[:, :, z] >= T2
    else:
        min_v = np.float32(sup.min())
        with np.errstate(all="ignore"):
            g = (sup - min_v) / np.float32(max_v - min_v)
        weak = (g >= np.float32(t1)) & (g < np.float32(t2))
        strong = g >= np.float32(t2)
    out = np.zeros((d0, d1, d2), np.int8, order="F")
    for z in range(d2):
        out[:, :, z] = canny_hysteresis(strong[:, :, z], weak[:, :, z])
    return out


# ---------------------------------------------------------------------------
# af_unwrap / af_wrap (public form: dilation 1, is_column, every type)
# ---------------------------------------------------------------------------
def patch_grid(W, H, wx, wy, sx, sy, px, py):
    """Patches across and down, with C's truncating division as the reference
    computes them (a window wider than the padded image by less than the stride
    still gives one patch)."""
    return (_cdiv_trunc(W + 2 * px - wx, sx) + 1, _cdiv_trunc(H + 2 * py - wy, sy) + 1)


def _patch_coords(nx, ny, wx, wy, sx, sy, px, py):
    """(x, y) image coordinates of every patch element, indexed [k, col] with
    k = kx + wx*ky and col = winx + nx*winy (src/backend/cpu/kernel/unwrap.hpp:40-71)."""
    k = np.arange(wx * wy)
    col = np.arange(nx * ny)
    x = (col % nx)[None, :] * sx - px + (k % wx)[:, None]
    y = (col // nx)[None, :] * sy - py + (k // wx)[:, None]
    return x, y


def unwrap_patches(sig: np.ndarray, wx, wy, sx, sy, px, py, is_column=True, dtype=None,
                   which="port") -> np.ndarray:
    """af_unwrap (src/api/c/unwrap.cpp:37-103, src/backend/cpu/unwrap.cpp:23-41)."""
    s = as_af(sig)
    sd = _dims4(s)
    nx, ny = patch_grid(sd[0], sd[1], wx, wy, sx, sy, px, py)
    if which == "ref":
        od = [wx * wy, nx * ny, sd[2], sd[3]] if is_column else [nx * ny, wx * wy, sd[2], sd[3]]
        out = np.zeros(od, dtype=s.dtype, order="F")
        rc = lib("ref").ref_unwrap_any(ctypes.c_int(dtype), out.ctypes.data_as(_P),
                                       s.ctypes.data_as(_P), _ll(sd),
                                       *[ctypes.c_longlong(v) for v in (wx, wy, sx, sy, px, py)],
                                       ctypes.c_int(1 if is_column else 0))
        if rc != 0:
            raise RuntimeError("ref_unwrap_any failed")
        return out
    x, y = _patch_coords(nx, ny, wx, wy, sx, sy, px, py)
    inside = (x >= 0) & (x < sd[0]) & (y >= 0) & (y < sd[1])
    cols = np.zeros([wx * wy, nx * ny, sd[2], sd[3]], dtype=s.dtype, order="F")
    cols[inside] = s[x[inside], y[inside]]
    return np.asfortranarray(cols if is_column else cols.transpose(1, 0, 2, 3))


def wrap_patches(cols: np.ndarray, ox, oy, wx, wy, sx, sy, px, py, is_column=True, out=None,
                 dtype=None, which="port") -> np.ndarray:
    """af_wrap / af_wrap_v2 (src/api/c/wrap.cpp:33-109, src/backend/cpu/kernel/wrap.hpp:21-80):
    out (zeros unless given) += every patch element, patches in increasing col
    order, each add in the element type."""
    c = as_af(cols)
    cd = _dims4(c)
    od = [ox, oy, cd[2], cd[3]]
    res = np.zeros(od, dtype=c.dtype, order="F") if out is None else np.array(as_af(out), order="F")
    nx, ny = patch_grid(ox, oy, wx, wy, sx, sy, px, py)
    if which == "ref":
        rc = lib("ref").ref_wrap_any(ctypes.c_int(dtype), res.ctypes.data_as(_P), _ll(od),
                                     c.ctypes.data_as(_P), _ll(cd),
                                     *[ctypes.c_longlong(v) for v in (wx, wy, sx, sy, px, py)],
                                     ctypes.c_int(1 if is_column else 0))
        if rc != 0:
            raise RuntimeError("ref_wrap_any failed")
        return res
    if nx < 0 or ny < 0:
        raise ValueError("window exceeds the padded image by a stride or more")
    km = c if is_column else c.transpose(1, 0, 2, 3)          # [k, col, d2, d3]
    x, y = _patch_coords(nx, ny, wx, wy, sx, sy, px, py)
    with np.errstate(over="ignore"):
        for col in range(nx * ny):
            m = (x[:, col] >= 0) & (x[:, col] < ox) & (y[:, col] >= 0) & (y[:, col] < oy)
            xs, ys = x[m, col], y[m, col]
            res[xs, ys] = res[xs, ys] + km[m, col]
    return res


# ---------------------------------------------------------------------------
# NN convolution, FP64
# ---------------------------------------------------------------------------
def _geom(sd, fd, stride, pad, dil):
    return _ll([sd[0], sd[1], sd[2], sd[3], fd[0], fd[1], fd[3], stride[0], stride[1],
                pad[0], pad[1], dil[0], dil[1]])


def _f64(a):
    return np.asfortranarray(as_af(a).astype(np.float64))


def nn_forward_f64(sig, filt, stride, pad, dil):
    s, f = _f64(sig), _f64(filt)
    sd, fd = _dims4(s), _dims4(f)
    od = nn_output_dims(sd, fd, stride, pad, dil)
    out = np.zeros(od, dtype=np.float64, order="F")
    lib().oracle_nn_fwd_f64(out.ctypes.data_as(_P), s.ctypes.data_as(_P), f.ctypes.data_as(_P),
                            _geom(sd, fd, stride, pad, dil))
    return out


def nn_forward_points_f64(sig, filt, stride, pad, dil, idx):
    s, f = _f64(sig), _f64(filt)
    sd, fd = _dims4(s), _dims4(f)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    vals = np.zeros(idx.size, dtype=np.float64)
    lib().oracle_nn_fwd_points_f64(vals.ctypes.data_as(_P), idx.ctypes.data_as(_P),
                                   ctypes.c_longlong(idx.size), s.ctypes.data_as(_P),
                                   f.ctypes.data_as(_P), _geom(sd, fd, stride, pad, dil))
    return vals


def nn_data_grad_f64(grad, sig_dims, filt, stride, pad, dil):
    g, f = _f64(grad), _f64(filt)
    fd = _dims4(f)
    sd = list(sig_dims)
    out = np.zeros(sd, dtype=np.float64, order="F")
    lib().oracle_nn_dgrad_f64(out.ctypes.data_as(_P), g.ctypes.data_as(_P), f.ctypes.data_as(_P),
                              _geom(sd, fd, stride, pad, dil))
    return out


def nn_data_grad_points_f64(grad, sig_dims, filt, stride, pad, dil, idx):
    g, f = _f64(grad), _f64(filt)
    fd = _dims4(f)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    vals = np.zeros(idx.size, dtype=np.float64)
    lib().oracle_nn_dgrad_points_f64(vals.ctypes.data_as(_P), idx.ctypes.data_as(_P),
                                     ctypes.c_longlong(idx.size), g.ctypes.data_as(_P),
                                     f.ctypes.data_as(_P), _geom(list(sig_dims), fd, stride, pad, dil))
    return vals


def nn_filter_grad_f64(grad, sig, filt_dims, stride, pad, dil):
    g, s = _f64(grad), _f64(sig)
    sd = _dims4(s)
    fd = list(filt_dims)
    out = np.zeros(fd, dtype=np.float64, order="F")
    lib().oracle_nn_wgrad_f64(out.ctypes.data_as(_P), s.ctypes.data_as(_P), g.ctypes.data_as(_P),
                              _geom(sd, fd, stride, pad, dil))
    return out


def nn_filter_grad_points_f64(grad, sig, filt_dims, stride, pad, dil, idx):
    g, s = _f64(grad), _f64(sig)
    sd = _dims4(s)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    vals = np.zeros(idx.size, dtype=np.float64)
    lib().oracle_nn_wgrad_points_f64(vals.ctypes.data_as(_P), idx.ctypes.data_as(_P),
                                     ctypes.c_longlong(idx.size), s.ctypes.data_as(_P),
                                     g.ctypes.data_as(_P), _geom(sd, list(filt_dims), stride, pad, dil))
    return vals


def nn_bias_grad_f64(grad, sig_dims, filt_dims, stride, pad, dil):
    g = _f64(grad)
    out = np.zeros([1, 1, filt_dims[3], 1], dtype=np.float64, order="F")
    lib().oracle_nn_bgrad_f64(out.ctypes.data_as(_P), g.ctypes.data_as(_P),
                              _geom(list(sig_dims), list(filt_dims), stride, pad, dil))
    return out


# ---------------------------------------------------------------------------
# the reference CPU backend's NN path, FP32: unwrap + GEMM
# (src/backend/cpu/convolve.cpp:123-158).  Used as the timed CPU baseline; the
# GEMM is numpy's bundled BLAS sgemm, standing in for the CBLAS call of
# src/backend/cpu/blas.cpp:222-331.
# ---------------------------------------------------------------------------
def nn_forward_unwrap_gemm_f32(sig, filt, stride, pad, dil, which="port"):
    s = as_af(sig, np.float32)
    f = as_af(filt, np.float32)
    sd, fd = _dims4(s), _dims4(f)
    od = nn_output_dims(sd, fd, stride, pad, dil)
    cols = unwrap(s, fd[0], fd[1], stride[0], stride[1], pad[0], pad[1], dil[0], dil[1], which)
    wsz, npix, C, N = cols.shape  # cols[tap, pixel, c, n], tap = x + fw*y
    A = np.ascontiguousarray(cols.transpose(1, 3, 2, 0)).reshape(npix * N, C * wsz)
    wflip = f[::-1, ::-1, :, :]  # flip(filter, {1,1,0,0})
    B = np.ascontiguousarray(
        wflip.reshape(wsz, C, fd[3], order="F").transpose(1, 0, 2)).reshape(C * wsz, fd[3])
    res = (A @ B).reshape(npix, N, fd[3]).transpose(0, 2, 1)  # (pixel, K, N)
    return np.asfortranarray(res).reshape(od, order="F")
