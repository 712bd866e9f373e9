"""Generate the golden fixtures from the reference's own CPU kernels.

Run here (where the ArrayFire v3.10.0 source tree is available):

    make -C oracle port ref
    python tests/golden/gen_golden.py

Writes, next to this file:
  direct.json  SHA-256 of the reference output bytes for every direct
               convolution case (tests/golden/cases.py:direct_cases) and the
               two full-size image workloads (512x512 Gaussian, 1024x1024
               neighbour count);
  sep.json     the same for af_convolve2_sep cases;
  patches.json SHA-256 of the reference's af_unwrap output, af_wrap of a
               seeded patch matrix into zeros, and af_wrap_v2 into a seeded
               image, for every tests/golden/cases.py:patch_cases case;
  image.json   SHA-256 of the reference's Sobel derivatives (dx, dy) for every
               tests/golden/cases.py:sobel_cases case;
  harris.json  the count and SHA-256 of x, y and score of the reference's
               Harris corners for every tests/golden/cases.py:harris_cases
               case (its CPU kernels composed as its CPU backend does);
  canny.json   the edge count and SHA-256 of the reference's Canny edge map
               for every tests/golden/cases.py:canny_cases case;
  nn.npz       FP64 NN forward / data-gradient / filter-gradient outputs for
               NN_CASES, each cross-checked against the reference's own
               unwrap + GEMM (forward, filter gradient) and wrap_dilated
               (data gradient) before it is written.

The oracle port (oracle/conv_oracle.c) is asserted bit-identical to the
reference for every direct/separable case while generating, so the fixtures
also record that the port was pinned.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import oracle as O  # noqa: E402
import cases as C  # noqa: E402


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def patches() -> None:
    """af_unwrap / af_wrap / af_wrap_v2 digests from the reference kernels,
    with the numpy port asserted bit-identical on every case."""
    gold = {}
    for case in C.patch_cases():
        cid, dt, sd, wx, wy, sx, sy, px, py, col, seed = case
        img = C.patch_values(dt, sd, seed)
        geo = (wx, wy, sx, sy, px, py, col)
        u_ref = O.unwrap_patches(img, *geo, dtype=dt, which="ref")
        u_port = O.unwrap_patches(img, *geo, dtype=dt, which="port")
        pm = C.patch_values(dt, C.patch_dims(case), seed + 1)
        base = C.patch_values(dt, sd, seed + 2)
        w_ref = O.wrap_patches(pm, sd[0], sd[1], *geo, dtype=dt, which="ref")
        w_port = O.wrap_patches(pm, sd[0], sd[1], *geo, dtype=dt, which="port")
        v_ref = O.wrap_patches(pm, sd[0], sd[1], *geo, out=base, dtype=dt, which="ref")
        v_port = O.wrap_patches(pm, sd[0], sd[1], *geo, out=base, dtype=dt, which="port")
        for name, a, b in (("unwrap", u_ref, u_port), ("wrap", w_ref, w_port),
                           ("wrap_v2", v_ref, v_port)):
            if a.shape != b.shape or a.tobytes(order="F") != b.tobytes(order="F"):
                raise SystemExit(f"port differs from reference on {cid} {name}")
        gold[cid] = {"unwrap": digest(u_ref), "unwrap_dims": list(u_ref.shape),
                     "wrap": digest(w_ref), "wrap_v2": digest(v_ref)}
    (HERE / "patches.json").write_text(json.dumps(gold, indent=0, sort_keys=True))
    print(f"patches {len(gold)}")


def images() -> None:
    """af_sobel_operator digests from the reference's CPU kernel, with the
    numpy port asserted bit-identical on every case."""
    gold = {}
    for cid, dt, shape, seed in C.sobel_cases():
        x = C.sobel_input(dt, shape, seed)
        rx, ry = O.sobel(x, dt, which="ref")
        px, py = O.sobel(x, dt, which="port")
        if rx.tobytes(order="F") != px.tobytes(order="F") or \
                ry.tobytes(order="F") != py.tobytes(order="F"):
            raise SystemExit(f"port differs from reference on {cid}")
        gold[cid] = {"dx": digest(rx), "dy": digest(ry)}
    (HERE / "image.json").write_text(json.dumps(gold, indent=0, sort_keys=True))
    print(f"image {len(gold)}")


def harris() -> None:
    """af_harris corners (count, x, y, score) from the reference's CPU
    kernels composed as src/backend/cpu/harris.cpp does, with the numpy port
    asserted bit-identical on every case."""
    gold = {}
    for cid, dt, shape, mc, mr, sg, bs, k, kind, seed in C.harris_cases():
        img = C.harris_image(dt, shape, kind, seed)
        ref = O.harris(img, dt, mc, mr, sg, bs, k, which="ref")
        port = O.harris(img, dt, mc, mr, sg, bs, k, which="port")
        if any(a.tobytes() != b.tobytes() for a, b in zip(ref, port)):
            raise SystemExit(f"port differs from reference on {cid}")
        gold[cid] = {"n": int(ref[0].size), "x": digest(ref[0]), "y": digest(ref[1]),
                     "score": digest(ref[2])}
    (HERE / "harris.json").write_text(json.dumps(gold, indent=0, sort_keys=True))
    print(f"harris {len(gold)}")


def canny() -> None:
    """af_canny edge maps from the reference's CPU kernels composed as
    src/api/c/canny.cpp does, with the numpy port asserted bit-identical on
    every case."""
    gold = {}
    for cid, dt, shape, otsu, t1, t2, isf, kind, seed in C.canny_cases():
        img = C.canny_image(dt, shape, kind, seed)
        ref = O.canny(img, dt, otsu, t1, t2, isf, which="ref")
        port = O.canny(img, dt, otsu, t1, t2, isf)
        if ref.tobytes(order="F") != port.tobytes(order="F"):
            raise SystemExit(f"port differs from reference on {cid}")
        gold[cid] = {"edges": int(ref.sum()), "digest": digest(ref)}
    (HERE / "canny.json").write_text(json.dumps(gold, indent=0, sort_keys=True))
    print(f"canny {len(gold)}")


def main() -> None:
    if O.build_ref() is None:
        raise SystemExit("reference source tree not found; golden vectors need it")
    O.build_port()

    direct = {}
    for cid, dt, rank, sd, fd, expand, seed in C.direct_cases():
        s = C.make_signal(dt, sd, seed)
        f = C.make_filter(dt, fd, seed + 1, rank)
        ref = O.convolve(s, f, dt, rank, expand, "ref")
        port = O.convolve(s, f, dt, rank, expand, "port")
        if ref.tobytes() != port.tobytes():
            raise SystemExit(f"port differs from reference on {cid}")
        direct[cid] = {"sha256": digest(ref), "dims": list(ref.shape)}
    for name, fn in (("config1a_gauss5_512", C.config1a), ("config1b_neighbour3_1024", C.config1b)):
        s, f = fn()
        ref = O.convolve(s, f, C.F32, 2, False, "ref")
        port = O.convolve(s, f, C.F32, 2, False, "port")
        if ref.tobytes() != port.tobytes():
            raise SystemExit(f"port differs from reference on {name}")
        direct[name] = {"sha256": digest(ref), "dims": list(ref.shape)}
    (HERE / "direct.json").write_text(json.dumps(direct, indent=0, sort_keys=True))

    sep = {}
    for cid, dt, sd, cl, rl, expand, seed in C.sep_cases():
        s = C.sep_signal(dt, sd, seed)
        cf = C.sep_taps(dt, cl, seed + 1)
        rf = C.sep_taps(dt, rl, seed + 2)
        ref = O.convolve2_sep(s, cf, rf, dt, expand, "ref")
        port = O.convolve2_sep(s, cf, rf, dt, expand, "port")
        if ref.tobytes() != port.tobytes():
            raise SystemExit(f"port differs from reference on {cid}")
        sep[cid] = {"sha256": digest(ref), "dims": list(ref.shape)}
    (HERE / "sep.json").write_text(json.dumps(sep, indent=0, sort_keys=True))

    # NN: FP64 direct loops, pinned to the reference's unwrap / wrap_dilated
    arrays = {}
    for i, case in enumerate(C.NN_CASES):
        name, sd, fd, st, pd, dl = case
        s, f = C.nn_inputs(case, 9000 + 10 * i, np.float64)
        g = C.nn_grad(case, 9000 + 10 * i, np.float64)
        fwd = O.nn_forward_f64(s, f, st, pd, dl)
        # reference path: unwrap (ref kernel) + FP64 GEMM with the flipped filter
        cols = O.unwrap(s, fd[0], fd[1], st[0], st[1], pd[0], pd[1], dl[0], dl[1], "ref")
        wsz, npix, Cc, N = cols.shape
        A = np.ascontiguousarray(cols.transpose(1, 3, 2, 0)).reshape(npix * N, Cc * wsz)
        wflip = f[::-1, ::-1, :, :]
        B = np.ascontiguousarray(wflip.reshape(wsz, Cc, fd[3], order="F").transpose(1, 0, 2)
                                 ).reshape(Cc * wsz, fd[3])
        ref_fwd = np.asfortranarray((A @ B).reshape(npix, N, fd[3]).transpose(0, 2, 1)).reshape(
            fwd.shape, order="F")
        assert np.allclose(fwd, ref_fwd, rtol=1e-12, atol=1e-12), name
        # filter gradient: unwrap^T * G, flipped (src/backend/cpu/convolve.cpp:213-243)
        G = np.ascontiguousarray(g.transpose(0, 1, 3, 2)).reshape(-1, fd[3], order="F")
        # rows of A must follow G's (pixel, n) order: pixel fastest then n
        A2 = np.ascontiguousarray(cols.transpose(1, 3, 2, 0)).reshape(npix, N, Cc * wsz)
        A2 = A2.transpose(1, 0, 2).reshape(N * npix, Cc * wsz)  # row = n*npix + pixel
        G2 = np.asfortranarray(g).reshape(npix, fd[3], N, order="F").transpose(2, 0, 1).reshape(
            N * npix, fd[3])
        R = A2.T @ G2  # ((c,tap), K)
        res = R.reshape(Cc, wsz, fd[3]).transpose(1, 0, 2).reshape(fd[0], fd[1], Cc, fd[3],
                                                                      order="F")
        ref_wgrad = np.asfortranarray(res[::-1, ::-1, :, :])
        wgrad = O.nn_filter_grad_f64(g, s, list(f.shape), st, pd, dl)
        assert np.allclose(wgrad, ref_wgrad, rtol=1e-12, atol=1e-12), name
        del G
        # data gradient: G * flip(W)^T then the reference's wrap_dilated
        colsg = (G2 @ B.T)  # rows n*npix+pixel, cols (c, tap)
        colsg = colsg.reshape(N, npix, Cc, wsz).transpose(3, 1, 2, 0)  # (tap, pixel, c, n)
        ref_dgrad = O.wrap_dilated(np.asfortranarray(colsg), list(s.shape), fd[0], fd[1], st[0],
                                   st[1], pd[0], pd[1], dl[0], dl[1], "ref")
        dgrad = O.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl)
        assert np.allclose(dgrad, ref_dgrad, rtol=1e-12, atol=1e-12), name
        arrays[f"{name}__fwd"] = fwd
        arrays[f"{name}__dgrad"] = dgrad
        arrays[f"{name}__wgrad"] = wgrad
    np.savez_compressed(HERE / "nn.npz", **arrays)
    print(f"direct {len(direct)}  sep {len(sep)}  nn {len(arrays)}")


if __name__ == "__main__":
    parts = {"patches": patches, "images": images, "harris": harris, "canny": canny}
    if sys.argv[1:] and all(a in parts for a in sys.argv[1:]):
        if O.build_ref() is None:
            raise SystemExit("reference source tree not found; golden vectors need it")
        for a in sys.argv[1:]:
            parts[a]()
    else:
        main()
        patches()
        images()
        harris()
        canny()
