"""The allocation-free entry point dk_build_environment_samples_noalloc.

Some callers of this library cannot let it call cudaMalloc: applications that
hand the renderer only device memory from their own arena or pool, and real-
time frame loops that must not allocate.  For them the environment-table
builder has a variant whose FP64 scratch is one static __device__ array of at
most DK_ENV_NOALLOC_MAX_TEXELS texels; the caller passes device pointers for
the texels and the table.  This file checks, through the C ABI, that the
variant produces the same table as the allocating entry point on consecutive
calls (which share and overwrite the one scratch array), and that it rejects
maps larger than its scratch.  It is collected last so that a failure here
leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from denrimrendererkit_gb300 import abi, library, scenes
from denrimrendererkit_gb300.scene import Texture2D

pytestmark = pytest.mark.gpu

MAX_TEXELS = 2048 * 1024  # DK_ENV_NOALLOC_MAX_TEXELS in include/denrim_cuda.h


def noalloc_table(lib, torch, tex, intensity, max_radiance):
    px = torch.from_numpy(np.ascontiguousarray(np.asarray(tex.pixels, np.float32).reshape(-1, 4))).cuda()
    out = torch.full((tex.width * tex.height, 2), -1.0, dtype=torch.float32, device="cuda")
    count = C.c_uint32(12345)
    torch.cuda.synchronize()
    rc = lib.dk_build_environment_samples_noalloc(px.data_ptr(), tex.width, tex.height, intensity, max_radiance,
                                                  out.data_ptr(), C.byref(count), None)
    library.check(rc)
    table = out.cpu().numpy().view(np.float32).reshape(-1, 2)[: count.value]
    return table.copy(), count.value


def allocating_table(tex, intensity, max_radiance):
    t = library.build_environment_samples(tex, intensity, max_radiance)
    return np.stack([t["cdf"], t["pdf_solid_angle"]], axis=-1), len(t)


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(dk_lib):
    torch = pytest.importorskip("torch")
    lib = library.load()
    library.check(lib.dk_device_open(0))
    maps = [(scenes.synthetic_hdri(512, 256, seed=3), 1.0, 0.0),
            (scenes.synthetic_hdri(2048, 1024, seed=4), 0.7, 16.0),  # exactly the maximum size
            (scenes.synthetic_hdri(512, 256, seed=3), 1.0, 0.0)]
    for tex, intensity, max_r in maps:
        want, n_want = allocating_table(tex, intensity, max_r)
        got, n_got = noalloc_table(lib, torch, tex, intensity, max_r)
        assert n_got == n_want == tex.width * tex.height
        # Same FP64 arithmetic on both sides; tolerance as the table tests use.
        np.testing.assert_allclose(got[:, 0], want[:, 0], rtol=0, atol=1e-6)
        np.testing.assert_allclose(got[:, 1], want[:, 1], rtol=1e-6, atol=1e-9)
        assert got[-1, 0] == 1.0


def test_noalloc_small_known_answer_and_empty_map(dk_lib):
    torch = pytest.importorskip("torch")
    lib = library.load()
    library.check(lib.dk_device_open(0))
    small = Texture2D(2, 1, np.array([[1, 1, 1, 1], [3, 3, 3, 1]], np.float32), 1)
    got, n = noalloc_table(lib, torch, small, 1.0, 0.0)
    assert n == 2 and got[:, 0].tolist() == pytest.approx([0.25, 1.0], abs=1e-6)  # BVHFlattenerTests.swift:153-183
    dark = Texture2D(4, 2, np.zeros((8, 4), np.float32), 1)
    _, n = noalloc_table(lib, torch, dark, 1.0, 0.0)
    assert n == 0


def test_noalloc_rejects_maps_beyond_the_scratch(dk_lib):
    torch = pytest.importorskip("torch")
    lib = library.load()
    library.check(lib.dk_device_open(0))
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    count = C.c_uint32(7)
    rc = lib.dk_build_environment_samples_noalloc(buf.data_ptr(), 2048, 1025, 1.0, 0.0, buf.data_ptr(),
                                                  C.byref(count), None)
    assert rc == 6  # DK_ERROR_INVALID_ARGUMENT, checked before any device work
    assert count.value == 0
    assert b"DK_ENV_NOALLOC_MAX_TEXELS" in lib.dk_last_error_message()


def test_noalloc_rejects_host_and_misaligned_pointers(dk_lib):
    # Both are refused on the host before any device work: a kernel never
    # sees such a pointer.
    torch = pytest.importorskip("torch")
    lib = library.load()
    library.check(lib.dk_device_open(0))
    dev = torch.zeros(64, dtype=torch.float32, device="cuda")
    host = np.zeros(64, np.float32)
    count = C.c_uint32(7)
    cases = [(dev.data_ptr() + 4, dev.data_ptr()),      # texels not 16-byte aligned
             (dev.data_ptr(), dev.data_ptr() + 4),      # table not 8-byte aligned
             (host.ctypes.data, dev.data_ptr()),        # texels in host memory
             (dev.data_ptr(), host.ctypes.data)]        # table in host memory
    for px, out in cases:
        rc = lib.dk_build_environment_samples_noalloc(px, 2, 2, 1.0, 0.0, out, C.byref(count), None)
        assert rc == 6 and count.value == 0
    assert np.all(host == 0)
