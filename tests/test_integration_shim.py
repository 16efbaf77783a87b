"""The C++ RenderPass binding a host application adds (tests/integration/
wavefront_gb300_pass.h over include/krr_wavefront_pass.hpp), compiled with
g++ against stand-ins for the host's RenderPass types and linked to
libkrr_gb300.so.  On the CPU: the pass is made by name from its JSON
parameters through the host's factory.  On the GPU: frames rendered through
the host's RenderPass virtuals equal the Python front end's bit for bit."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from kiraray_gb300 import _lib, scenes

ROOT = Path(__file__).resolve().parents[1]
HERE = Path(__file__).resolve().parent / "integration"


@pytest.fixture(scope="module")
def shim(krr_lib, tmp_path_factory):
    out = tmp_path_factory.mktemp("shim") / "libpass_shim.so"
    lib_dir = _lib.LIB_PATH.parent
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-shared", "-fPIC",
           "-I", str(ROOT / "include"), "-I", str(HERE), str(HERE / "pass_shim.cpp"),
           "-o", str(out), "-L", str(lib_dir), "-lkrr_gb300", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(out))
    lib.shim_params.argtypes = [C.c_char_p, C.POINTER(_lib.WfParams), C.c_char_p, C.c_int]
    lib.shim_render.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                C.c_void_p]
    return lib


def test_pass_made_by_name_from_json(shim):
    p = _lib.WfParams()
    name = C.create_string_buffer(64)
    assert shim.shim_params(b'{"max_depth": 4, "nee": false, "rr": 0.5}', C.byref(p), name, 64) == 0
    assert name.value == b"WavefrontPathTracer"
    assert (p.max_depth, p.nee, p.enable_medium) == (4, 0, 1) and p.rr == pytest.approx(0.5)
    assert shim.shim_params(b'{"max_depth": "four"}', C.byref(p), name, 64) == 1


@pytest.mark.gpu
def test_frames_through_the_renderpass_interface(shim, cuda):
    import torch
    from kiraray_gb300.wavefront import WavefrontPathTracer
    sc = scenes.cornell_box(64, 48, max_depth=4)
    desc, keep = sc.desc()
    cam = sc.camera.desc()
    out = torch.zeros((48, 64, 4), device="cuda")
    st = shim.shim_render(b'{"max_depth": 4}', C.addressof(desc), C.addressof(cam), 64, 48, 3,
                          out.data_ptr())
    torch.cuda.synchronize()
    assert st == 0
    pt = WavefrontPathTracer({"max_depth": 4})
    pt.set_scene(sc)
    pt.resize(64, 48)
    pt.begin_frame(3, sc.camera)
    want = pt.render().cpu().numpy()
    got = out.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert (got[..., :3] > 0).mean() > 0.3
