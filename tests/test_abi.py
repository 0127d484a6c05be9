"""The C ABI of libpico_gpu.so, checked without a GPU.

The library must load on a machine with no device, export every entry point
include/pico_gpu.h declares, bind each of them in the Python handles, and
answer the host-only calls (status strings, size bounds, argument checks,
initialisation without a device) without touching a GPU.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

import pico_gb300
from pico_gb300 import build

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(pico_gpu_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    build.build()
    return pico_gb300.load_library()


def test_every_declared_symbol_is_exported_and_bound(lib):
    names = declared_symbols()
    assert len(names) >= 20
    raw = C.CDLL(str(pico_gb300.LIB_PATH))
    missing = [n for n in sorted(names) if not hasattr(raw, n)]
    assert not missing, f"not exported: {missing}"
    unbound = sorted(names - set(pico_gb300.SIGNATURES))
    assert not unbound, f"declared but not bound in pico_gb300.SIGNATURES: {unbound}"
    extra = sorted(set(pico_gb300.SIGNATURES) - names)
    assert not extra, f"bound but not declared: {extra}"


def test_status_strings(lib):
    for code, name in pico_gb300.STATUS_NAMES.items():
        s = lib.pico_gpu_status_string(code)
        assert s and len(s) >= 2, name
    assert lib.pico_gpu_status_string(12345)


def test_hdr_bound_covers_worst_case(lib):
    # run-length coded scanlines: 4 header bytes + 4 components of W literals in runs of 128
    for w, h in [(1, 1), (7, 3), (8, 2), (128, 1), (129, 5), (1920, 1080), (40000, 2)]:
        bound = lib.pico_gpu_hdr_bound(w, h)
        rle = 8 <= w < 32768
        body = h * (4 + 4 * (w + (w + 127) // 128)) if rle else 4 * w * h
        assert bound >= 100 + body, (w, h)


def test_null_arguments_are_rejected(lib):
    n = C.c_size_t(0)
    assert lib.pico_gpu_encode_hdr(None, None, 4, 4, None, 0, C.byref(n)) == -1
    assert lib.pico_gpu_set_traversal_order(None, 0) == -1
    assert lib.pico_gpu_init(0, None) == -1
    assert lib.pico_gpu_last_error(None) is not None


def test_init_without_a_device_fails_cleanly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; this checks the no-device path")
    h = C.c_void_p()
    st = lib.pico_gpu_init(0, C.byref(h))
    assert st in (-7, -2), st
    assert not h.value


@pytest.mark.parametrize("prefix", ["cornell", "field"])
def test_product_sah_matches_the_reference_node_for_node(lib, prefix):
    """The BVHs pico_gpu_scene_upload builds (before flattening) equal the reference's own
    BVH<T,2> nodes, generated from the reference's code (tests/golden/trace.npz): the same
    boxes bit for bit, children, leaf ranges and leaf items, for every BLAS and the TLAS."""
    import sys
    import numpy as np
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from scene_io import load_scene
    z = np.load(ROOT / "tests" / "golden" / "trace.npz")
    scene = load_scene(z, prefix)
    trees = [(f"{prefix}_blas{mi}", mi) for mi in range(len(scene.meshes))] + [(f"{prefix}_tlas", -1)]
    for key, which in trees:
        boxes, links, values = pico_gb300.reference_bvh(scene, which)
        np.testing.assert_array_equal(boxes.view(np.uint32), z[f"{key}_boxes"].view(np.uint32), err_msg=key)
        np.testing.assert_array_equal(links, z[f"{key}_links"], err_msg=key)
        np.testing.assert_array_equal(values, z[f"{key}_values"], err_msg=key)
