"""Shared test setup: the gpu marker, import paths, and session fixtures that
build the library and the oracle if they are missing."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "patchvvc-plus_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def pvvc_lib():
    import pvvc
    pvvc.build_library()
    pvvc.lib()
    return pvvc


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import Reference, build_reference
    if build_reference() is None:
        pytest.skip("reference sources not present on this machine")
    return Reference()


def golden_frames(variant: str = "raw") -> list[bytes]:
    return [open(os.path.join(GOLDEN, "gop", f"{variant}_{f}.frame"), "rb").read() for f in range(4)]


def golden_expected():
    return np.load(os.path.join(GOLDEN, "gop", "expected.npz"))


def round_away(x: np.ndarray) -> np.ndarray:
    """std::round (half away from zero), exact for float32 inputs."""
    d = x.astype(np.float64)
    return np.sign(d) * np.floor(np.abs(d) + 0.5)


def rgb_precast(yuv: np.ndarray) -> np.ndarray:
    """The rounded floats ColorYUV::ConvertRGB casts to uint8 (float32 ops,
    left to right, include/common/common.h:154-158)."""
    f = np.float32
    y, u, v = yuv[:, 0].astype(f), yuv[:, 1].astype(f), yuv[:, 2].astype(f)
    r = y + f(1.402) * (v - f(128))
    g = (y - f(0.3441) * (u - f(128))) - f(0.7141) * (v - f(128))
    b = y + f(1.772) * (u - f(128))
    return round_away(np.stack([r, g, b], 1).astype(np.float32))


def rgb_matches(got: np.ndarray, ref_rgb: np.ndarray, oracle_yuv: np.ndarray) -> np.ndarray:
    """Per-point colour agreement.  Where the pre-cast float of
    ColorYUV::ConvertRGB (include/common/common.h:154-158) lies in [0, 255]
    the reference's uint8 cast is defined and the colour must equal the
    reference's; elsewhere the cast is undefined in the reference (it wraps on
    x86) and the product clamps, so the colour must equal the clamped value."""
    pre = rgb_precast(oracle_yuv)
    inrange = (pre >= 0) & (pre <= 255)
    clamped = np.clip(pre, 0, 255).astype(np.uint8)
    want = np.where(inrange, ref_rgb, clamped)
    return got == want
