"""CPU tests of the image-op oracles: the Sobel port against the digests of
the reference's own CPU kernel (tests/golden/image.json, written by
tests/golden/gen_golden.py with the port asserted identical), and the
Gaussian against its closed form and the reference's documented defaults."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "image.json").read_text())


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


@pytest.mark.parametrize("case", C.sobel_cases(), ids=lambda c: c[0])
def test_sobel_port_matches_reference_hash(oracle, case):
    cid, dt, shape, seed = case
    dx, dy = oracle.sobel(C.sobel_input(dt, shape, seed), dt)
    assert digest(dx) == GOLD[cid]["dx"]
    assert digest(dy) == GOLD[cid]["dy"]


def test_gaussian_oracle_closed_form(oracle):
    g = oracle.gaussian_kernel(5, 5, 1.0, 1.0)
    x = np.arange(5) - 2
    k = np.exp(-0.5 * (x[:, None] ** 2 + x[None, :] ** 2))
    np.testing.assert_allclose(g, k / k.sum(), rtol=1e-14)
    # sigma <= 0 means a quarter of the size; a single row or column is 1-D
    g = oracle.gaussian_kernel(1, 8)
    x = (np.arange(8) - 3.5) / 2.0
    k = np.exp(-0.5 * x ** 2)
    np.testing.assert_allclose(g[0], k / k.sum(), rtol=1e-14)
    assert abs(oracle.gaussian_kernel(7, 3, 0.7, 2.0).sum() - 1) < 1e-14


def test_dog_oracle_is_blur_difference(oracle):
    img = np.asfortranarray(np.ones((20, 16), np.float32))
    d = oracle.dog(img, C.F32, 3, 2)
    # a constant image blurred by unit-sum kernels is unchanged away from the
    # zero-padded borders, so the difference vanishes in the interior
    assert np.abs(d[3:-3, 3:-3]).max() < 1e-6
